/*
 * simkit_gb300: C ABI of the GB300 backward-Euler stable neo-Hookean FEM path.
 *
 * The reference (otmanon/simkit) is a pure-Python library; its "interface"
 * for this path is a set of Python functions over numpy arrays and scipy
 * sparse matrices.  Each entry point below replaces one of them (or the
 * numpy/scipy work inside one of them) and cites it as file:line within the
 * simkit project.  The Python package simkit_gb300 binds these with ctypes
 * and keeps simkit's Python signatures on top.
 *
 * Conventions
 *   - Every pointer argument is a DEVICE pointer unless its name ends in _h
 *     (host).  The caller owns all memory: nothing here allocates device
 *     memory.  Entry points that need scratch take a workspace pointer whose
 *     size a matching *_workspace_size() query returns.
 *   - `stream` is a cudaStream_t passed as void*; 0 is the legacy stream.
 *     Work is stream-ordered; entry points synchronize only where they must
 *     return a host scalar (documented per function).
 *   - Return value: 0 on success, a negative skg_status on failure;
 *     skg_last_error() returns the message of the calling thread's last error.
 *   - Positions are simkit's layout: x[3 i + c], float64 (simkit/deformation_jacobian.py:13-16).
 *   - Element tier F arrays are (t, d, d) row-major float64 (snh.py:65-129).
 */
#ifndef SIMKIT_GB300_H_
#define SIMKIT_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum skg_status {
  SKG_OK = 0,
  SKG_ERR_ARG = -1,        /* invalid argument (simkit raises ValueError) */
  SKG_ERR_CUDA = -2,       /* a CUDA runtime call failed */
  SKG_ERR_NOT_CONVERGED = -3,
  SKG_ERR_LINESEARCH = -4, /* Armijo search exhausted: simkit returns t = 0 (backtracking_line_search.py:66-67) */
  SKG_ERR_NONFINITE = -5,  /* NaN/Inf in an energy, gradient or residual */
  SKG_ERR_TIMEOUT = -6,    /* a bounded grid-wide wait gave up */
  SKG_ERR_CAPACITY = -7    /* a size exceeds a fixed capacity */
} skg_status;

typedef enum skg_precision {
  SKG_FP64 = 0,  /* every kernel in FP64 */
  SKG_MIXED = 1  /* FP32 element Hessians, SpMV and PCG vectors; FP64 gradient,
                    residual norms, dot products and energy sums */
} skg_precision;

/* ---------------------------------------------------------------------- */
/* errors / version                                                        */
/* ---------------------------------------------------------------------- */
int skg_version(void);
/* Copies the calling thread's last error message into buf (NUL-terminated). */
int skg_last_error(char* buf_h, size_t len);

/* ---------------------------------------------------------------------- */
/* element tier: simkit/energies/stable_neo_hookean.py                     */
/* ---------------------------------------------------------------------- */
/* psi per element.  Replaces stable_neo_hookean_energy_element_F (snh.py:65-129).
 * dim 2 or 3; F (t,d,d) f64, mu/lam (t) f64 -> psi (t) f64. precision selects the
 * arithmetic (inputs and outputs stay f64). */
int skg_snh_energy_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                             double* psi, int64_t t, void* stream);
/* PK1 per element.  Replaces stable_neo_hookean_gradient_element_F (snh.py:132-218). */
int skg_snh_gradient_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                               double* P, int64_t t, void* stream);
/* d*d x d*d Hessian per element, not projected.  Replaces
 * stable_neo_hookean_hessian_element_F (snh.py:221-443). */
int skg_snh_hessian_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                              double* H, int64_t t, void* stream);

/* ---------------------------------------------------------------------- */
/* element tier: simkit/energies/macklin_mueller_neo_hookean.py            */
/* ---------------------------------------------------------------------- */
/* Same arguments as the stable neo-Hookean element tier.  Replace
 * macklin_mueller_neo_hookean_energy_element_F (:66-122), _gradient_element_F (:125-185)
 * and _hessian_element_F (:188-443, not projected). */
int skg_mmnh_energy_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                              double* psi, int64_t t, void* stream);
int skg_mmnh_gradient_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                                double* P, int64_t t, void* stream);
int skg_mmnh_hessian_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                               double* H, int64_t t, void* stream);

/* ---------------------------------------------------------------------- */
/* element tier: simkit/energies/arap.py and simkit/energies/fcr.py         */
/* ---------------------------------------------------------------------- */
/* Same arguments as the stable neo-Hookean element tier (lam is read by the
 * fixed-corotated entries only; the ARAP entries accept lam = NULL).  R is the
 * rotation of the rotation-variant SVD (simkit/polar_svd.py:59-90), dR/dF the
 * closed form of simkit/rotation_gradient.py:12-70.  Replace
 * arap_energy_element_F (arap.py:71-91), arap_gradient_element_F (:94-114),
 * arap_hessian_element_F (:117-145, not projected), fcr_energy_element_F
 * (fcr.py:41-62), fcr_gradient_element_F (:65-125) and fcr_hessian_element_F
 * (:128-302, not projected). */
int skg_arap_energy_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                              double* psi, int64_t t, void* stream);
int skg_arap_gradient_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                                double* P, int64_t t, void* stream);
int skg_arap_hessian_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                               double* H, int64_t t, void* stream);
int skg_fcr_energy_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                             double* psi, int64_t t, void* stream);
int skg_fcr_gradient_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                               double* P, int64_t t, void* stream);
int skg_fcr_hessian_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                              double* H, int64_t t, void* stream);

/* element tier: simkit/energies/linear_elasticity.py.  Same arguments; replace
 * linear_elasticity_energy_element_F (:43-70), _gradient_element_F (:73-100) and
 * _hessian_element_F (:103-136, constant in F). */
int skg_le_energy_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                            double* psi, int64_t t, void* stream);
int skg_le_gradient_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                              double* P, int64_t t, void* stream);
int skg_le_hessian_element_F(int dim, int precision, const double* F, const double* mu, const double* lam,
                             double* H, int64_t t, void* stream);

/* ---------------------------------------------------------------------- */
/* contact springs: simkit/energies/contact_springs_plane.py:44-200        */
/* ---------------------------------------------------------------------- */
/* One contact plane of simkit's contact springs (simkit/energies/contact_springs_plane.py:44-200):
 * every vertex with (x - p) . n < 0 adds k w ((x - p) . n)^2 / 2 to the energy, w = its lumped mass
 * (simkit's M argument) or 1. */
typedef struct skg_contact_plane {
  double p[3];  /* a point of the plane */
  double n[3];  /* unit normal (the allowed side) */
  double k;     /* spring stiffness */
} skg_contact_plane;

#define SKG_MAX_PLANES 4

/* Per vertex of x (n,3) f64 against one plane, weights w = mass (n) or 1 when mass is null:
 * energy_v (n) = k w d^2 / 2, grad (3n) = k w d n, hdiag (9n) = k w n n^T (row-major 3x3),
 * under (n) = 1 where d = (x - p) . n < 0 (everything else 0).  Any output may be null.
 * Replaces contact_springs_plane_energy / _gradient / _hessian (:44-200). */
int skg_contact_plane_terms(const double* x, int64_t n, const skg_contact_plane* plane_h, const double* mass,
                            double* energy_v, double* grad, double* hdiag, uint8_t* under, void* stream);

/* ---------------------------------------------------------------------- */
/* psd_project: simkit/psd_project.py:12-47                                */
/* ---------------------------------------------------------------------- */
/* Batched eigenvalue floor of symmetric d x d blocks (1 <= d <= 12) by cyclic
 * Jacobi.  method 0 = 'proj' (floor at 1e-6, :37), 1 = 'abs' (:35).
 * H and out may alias. */
int skg_psd_project(const double* H, double* out, int64_t n, int d, int method, void* stream);

/* ---------------------------------------------------------------------- */
/* mesh setup                                                              */
/* ---------------------------------------------------------------------- */
/* Per-tet inverse rest edge matrix Dinv (rows = grad N_1..3) and signed volume.
 * Replaces the per-element D of deformation_jacobian (deformation_jacobian.py:43-61)
 * and volume/tetrahedron_volumes (volume.py:14-41, tetrahedron_volumes.py:26-27).
 * X (n,3) f64, T (t,4) i32 -> dinv (9,t) f64 SoA, vol (t) f64.  A degenerate rest
 * tet gives non-finite Dinv entries (simkit's np.linalg.inv raises instead); a tet
 * with a vertex index outside [0, n) is not read and gets NaN vol and Dinv.  The
 * Python layer rejects both (ValueError) before any solve. */
int skg_tet_setup(const double* X, const int32_t* T, int64_t n, int64_t t, double* dinv, double* vol,
                  void* stream);

/* F = J x for the tet operator: F (t,3,3) f64 from positions x (3n) f64.
 * Replaces the sparse product J @ x (snh.py:499, deformation_jacobian.py example). */
int skg_tet_deformation_gradient(const int32_t* T, const double* dinv, const double* x, int64_t t,
                                 double* F, void* stream);
/* y = J^T vec(P): scatter-free vertex gather (deterministic). P (t,3,3) f64 -> y (3n) f64.
 * Replaces J.transpose() @ P.reshape(-1,1) (snh.py:501-502). */
int skg_tet_gradient_scatter(const int32_t* T, const double* dinv, const double* P, const int32_t* v2t_ptr,
                             const int32_t* v2t, int64_t n, int64_t t, double* y, void* stream);

/* Sparse pattern of K = J^T blockdiag(He) J for a tet mesh, as 3x3 blocks.
 * Host function (all pointers _h).  Pass 1 (rowptr == NULL): returns the number of
 * blocks in *n_blocks_h.  Pass 2 fills:
 *   bsr_rowptr (n+1), bsr_col (nb)  - block CSR, columns sorted ascending
 *   bsr_diag (n)                    - slot of each diagonal block
 *   hc_ptr (nb+1), hc_src (16 t)    - per slot, the per-tet blocks summed into it,
 *                                     encoded tet*16 + code, ordered by tet
 *   v2t_ptr (n+1), v2t (4 t)        - vertex -> (tet*4 + corner), ordered by tet
 * Expanded to scalars (row 3v+i, columns 3w+j) the block pattern equals the
 * pattern scipy produces for J.T @ block_diag(He) @ J (snh.py:536-537) whenever
 * no assembled entry cancels to exactly zero. */
int skg_pattern_build(const int32_t* T_h, int64_t n, int64_t t, int64_t* n_blocks_h, int32_t* bsr_rowptr_h,
                      int32_t* bsr_col_h, int32_t* bsr_diag_h, int32_t* hc_ptr_h, int32_t* hc_src_h,
                      int32_t* v2t_ptr_h, int32_t* v2t_h);

/* Mesh descriptor used by the assembled tier and the solver (all device pointers). */
/* Elastic energies of the per-tet kernels (simkit/energies/elastic.py:75 dispatches the same set
 * by name). */
typedef enum skg_material {
  SKG_MAT_STABLE_NEO_HOOKEAN = 0,          /* simkit/energies/stable_neo_hookean.py */
  SKG_MAT_MACKLIN_MUELLER_NEO_HOOKEAN = 1, /* simkit/energies/macklin_mueller_neo_hookean.py */
  SKG_MAT_ARAP = 2,                        /* simkit/energies/arap.py (lam unused) */
  SKG_MAT_FIXED_COROTATED = 3,             /* simkit/energies/fcr.py */
  SKG_MAT_LINEAR_ELASTICITY = 4            /* simkit/energies/linear_elasticity.py (Hessian never
                                              projected, as simkit's) */
} skg_material;

/* Two-level preconditioner data (optional; pcg_mode 7).  Vertices are grouped
 * into aggregates; each aggregate carries 6 coarse unknowns, 3 translations and
 * 3 rotations about its centroid, so (P e)_v = t_a + w_a x d_v on the free DOFs
 * of v.  The PCG preconditioner becomes D^-1 + P (P^T A P)^-1 P^T with D the
 * 3x3 block diagonal.  Built by the host from the rest positions, the pins and
 * the block pattern (simkit_gb300/mesh.py: coarse_aggregates).  simkit solves
 * the Newton systems with a direct solver (scipy spsolve in simkit/solvers/
 * newton.py:52); this preconditioner is the GPU's replacement for that
 * solver's robustness on stiff, heterogeneous meshes. */
typedef struct skg_coarse {
  int32_t n_agg;            /* aggregates; 6 n_agg coarse unknowns, at most 4096 in the whole-mesh form */
  int32_t n_cblocks;        /* nonzero 6x6 blocks of the coarse operator */
  const float* mode;        /* (n, 4) per vertex: (d_x, d_y, d_z, bits) with d the offset from the
                               aggregate centroid divided by the aggregate's RMS offset and bits
                               (as uint32) = aggregate | free-DOF mask << 29 (bit c: DOF c free) */
  const int32_t* cb_ptr;    /* (n_cblocks + 1) offsets into cb_slot */
  const int32_t* cb_slot;   /* (n_blocks) fine block slots grouped by coarse block */
  const int32_t* cb_rc;     /* (2 n_cblocks) aggregate row, aggregate column of each coarse block */
  /* Per-instance form, for the thread-block-cluster PCG (pcg_mode 2 / 3 on small meshes, and
   * skg_be_step_batched).  NULL inst_agg selects the whole-mesh form of pcg_mode 7.  Each
   * instance has at most 127 aggregates (762 coarse unknowns). */
  int32_t n_inst;           /* instances (1 for one mesh) */
  int32_t max_np;           /* largest 6 * aggregates of an instance, rounded up to 32 */
  int64_t m_floats;         /* sum over instances of np_i^2: dense coarse storage */
  const int32_t* inst_agg;  /* (n_inst + 1) first aggregate of each instance */
  const int32_t* agg_inst;  /* (n_agg) instance of each aggregate */
  const int64_t* inst_moff; /* (n_inst + 1) offset of each instance's np_i x np_i block, in floats */
  const uint32_t* colpack;  /* (n) per vertex: (k_x+64) | (k_y+64) << 7 | (k_z+64) << 14 | local
                               aggregate << 21 | free mask << 28, offset = k / 64 */
} skg_coarse;

typedef struct skg_tet_mesh {
  int64_t n_verts;
  int64_t n_tets;
  int64_t n_blocks;
  const int32_t* tets;       /* (t,4) */
  const double* dinv;        /* (9,t) SoA */
  const float* dinv32;       /* (9,t) SoA, FP32 copy (mixed precision) */
  const double* vol;         /* (t) signed rest volume */
  const double* mu;          /* (t) */
  const double* lam;         /* (t) */
  const float* mat32;        /* (3,t): vol, mu, lam in FP32 */
  const int32_t* bsr_rowptr; /* (n+1) */
  const int32_t* bsr_col;    /* (nb) */
  const int32_t* bsr_diag;   /* (n) slot of the diagonal block of each row */
  const int32_t* bsr_row;    /* (nb) block row of each slot */
  const int32_t* hc_ptr;     /* (nb+1) */
  const int32_t* hc_src;     /* (16t) */
  const int32_t* v2t_ptr;    /* (n+1) */
  const int32_t* v2t;        /* (4t) */
  int32_t material;          /* skg_material: the elastic energy of every tet */
  const skg_coarse* coarse;  /* host pointer to the two-level preconditioner data, or NULL */
  /* Optional upper-triangle lists (up_slot NULL: every slot is summed from hc_ptr / hc_src).  With
   * them the assembly sums each block (v, w), w >= v, once and writes its transpose into the slot
   * (w, v), so the assembled matrix is exactly symmetric and 10 instead of 16 per-tet blocks are
   * gathered per tet. */
  int64_t n_upper;           /* slots with column >= row */
  const int32_t* up_slot;    /* (n_upper) those slots, ascending */
  const int32_t* up_mirror;  /* (n_upper) slot of the transposed block (the slot itself on the diagonal) */
  const int32_t* hcu_ptr;    /* (n_upper+1) offsets into hcu_src */
  const int32_t* hcu_src;    /* contributions of the upper slots, encoded and ordered as hc_src */
} skg_tet_mesh;

/* Assembled block matrix (3x3 blocks).  Values of block slot s of row v live at
 * val[9*rowptr[v] + m*K_v + (s - rowptr[v])], m = 3i+j, K_v = rowptr[v+1]-rowptr[v]. */

/* ---------------------------------------------------------------------- */
/* assembled tier (x variable): snh.py:449-538                             */
/* ---------------------------------------------------------------------- */
/* Workspace bytes for the assembled-tier calls and the solver. */
int64_t skg_assembly_workspace_size(const skg_tet_mesh* mesh, int precision);

/* sum_e vol_e psi(F_e), F = J x.  Replaces stable_neo_hookean_energy_x (snh.py:449-474).
 * Synchronizes `stream` to return the value in *energy_h. */
int skg_snh_energy_x(const skg_tet_mesh* mesh, const double* x, double* energy_h, void* workspace,
                     void* stream);
/* J^T vec(vol P).  Replaces stable_neo_hookean_gradient_x (snh.py:477-503). g (3n) f64. */
int skg_snh_gradient_x(const skg_tet_mesh* mesh, const double* x, double* g, void* workspace, void* stream);
/* J^T blockdiag(psd(vol He)) J as block values.  Replaces stable_neo_hookean_hessian_x
 * (snh.py:506-538).  precision SKG_FP64 writes val64 (9 nb f64); SKG_MIXED writes val32.
 * psd != 0 applies simkit's 1e-6 eigenvalue floor to each vol-weighted 9x9 block. */
int skg_snh_hessian_x(const skg_tet_mesh* mesh, const double* x, int precision, int psd, double* val64,
                      float* val32, void* workspace, void* stream);

/* The displacement (_u) tier: F_e = (J u)_e + Jx_bar_e, where Jx_bar (9 t f64, row 9e + 3i + j =
 * F_ij, the layout of J's rows) is the caller's precomputed J x_bar for an arbitrary reference
 * x_bar.  Same outputs and workspace as the _x calls.  Replace stable_neo_hookean_energy_u
 * (snh.py:544-576), _gradient_u (:579-611) and _hessian_u (:614-648); with mesh->material they
 * also replace the _u functions of macklin_mueller_neo_hookean.py, arap.py and fcr.py. */
int skg_snh_energy_u(const skg_tet_mesh* mesh, const double* u, const double* Jx_bar, double* energy_h,
                     void* workspace, void* stream);
int skg_snh_gradient_u(const skg_tet_mesh* mesh, const double* u, const double* Jx_bar, double* g,
                       void* workspace, void* stream);
int skg_snh_hessian_u(const skg_tet_mesh* mesh, const double* u, const double* Jx_bar, int precision, int psd,
                      double* val64, float* val32, void* workspace, void* stream);

/* ---------------------------------------------------------------------- */
/* Newton / backward Euler: solvers/newton.py:7-75, integrators/backward_euler.py:27-91 */
/* ---------------------------------------------------------------------- */
/* Per-iteration record of one skg_be_step call, for simkit's newton_solver info dict
 * (solvers/newton.py:43-67: 'g', 'dx', 'alphas', 'iters'), plus the relative residual and the
 * PCG iterations of each Newton iteration.  Rows past newton_iters are left untouched. */
typedef struct skg_newton_record {
  int32_t capacity;         /* Newton iterations the arrays hold (>= max_newton to record all) */
  double* g;                /* device (capacity, 3n): gradient at the start of each iteration */
  double* dx;               /* device (capacity, 3n): Newton direction (solution of H dx = -g) */
  double* alpha_h;          /* host (capacity): accepted step length (0 when the search failed) */
  double* residual_h;       /* host (capacity): ||g|| / ||g(x_tilde)|| at the start of the iteration */
  int32_t* pcg_iters_h;     /* host (capacity): PCG iterations of the iteration's solve */
} skg_newton_record;

typedef struct skg_be_params {
  double dt;                /* time step h */
  double tol;               /* relative residual ||g(x)|| / ||g(x_tilde)|| */
  int32_t max_newton;       /* <= 20 in the standard workloads */
  int32_t precision;        /* skg_precision */
  double pcg_rtol;          /* PCG relative tolerance (forcing term) */
  int32_t pcg_max_iter;
  int32_t do_line_search;
  double ls_alpha;          /* Armijo parameter, simkit default 0.01 */
  double ls_beta;           /* step factor, simkit default 0.5 */
  int32_t ls_max_iter;      /* simkit default 100 */
  int32_t pcg_mode;         /* 0 kernel per phase, 1 grid-persistent cooperative kernel,
                               2 one thread-block cluster (two-level with the per-instance
                               coarse form), 3 by size (2 up to 24,576 block rows, else 7 with
                               the whole-mesh coarse form, else 5), 4 grid-persistent
                               Chronopoulos-Gear form, 5 grid-persistent with two barriers per
                               iteration, 7 grid-persistent two-level (needs the whole-mesh
                               coarse form; else 5) */
  double ls_threshold;      /* Armijo slack, simkit default 1e-12; < 0 selects a slack
                               scaled to the FP32 rounding of the energy sum */
  int32_t profile;          /* 1: time each phase with CUDA events (adds syncs) */
  int32_t pcg_variant;      /* grid-persistent PCG kernel variant 0-8 (lanes per row x rows in
                               flight: 8x1, 16x1, 8x2, 16x2, 4x2, 4x4, 2x4, 8x4, 2x2); for the
                               one-cluster PCG (mode 2) the cluster size: 0 by system size,
                               1-4 = 16, 8, 4, 2 CTAs; for the two-level grid PCG (mode 7) also
                               9-17 = the shapes of 0-8 with 768-thread blocks, and 18-20 = two
                               grid barriers per iteration instead of three (coarse residual by
                               recurrence), 768-thread blocks, shapes 4x2, 8x2, 2x2; chosen by the
                               autotuner */
  int32_t batch_min_cluster; /* batched PCG: smallest thread-block cluster an instance gets (1, 2,
                               4, 8 or 16; 0 = 4); each instance gets the smallest power of two
                               at least this large whose CTAs hold its vectors */
  int32_t batch_vec_kb;     /* batched PCG: the cluster size is the smallest whose per-CTA vectors
                               take at most this many KiB of shared memory, leaving the rest for
                               block records (0 = 170); if none does, the smallest that fits */
  int32_t integrator;       /* 0 backward Euler (simkit/integrators/backward_euler.py:27-91);
                               1 BDF2 (simkit/integrators/bdf2.py:31-101): target from four
                               displacement levels (simkit/energies/kinetic.py:93-101) and
                               kinetic factor 9/4; needs u_prev2 and u_prev3 */
  int32_t n_planes;         /* contact planes added to the potential (0..SKG_MAX_PLANES) */
  int32_t contact_mass_weighted; /* 1: spring weight = lumped vertex mass; 0: 1 */
  const skg_contact_plane* planes; /* host array of n_planes planes */
  int32_t coarse_refresh;   /* two-level PCG: rebuild the coarse inverse 0 = at the first Newton
                               iteration of this step, 1 = at every Newton iteration, -1 = not
                               at all: reuse the inverse an earlier call built in the same
                               workspace for the same mesh (the caller guarantees one exists) */
  int32_t stop_rule;        /* skg_be_step: 0 = relative residual ||g|| / ||g(x_tilde)|| < tol
                               (SKG_ERR_NOT_CONVERGED after max_newton); 1 = simkit's newton_solver
                               (solvers/newton.py:43-75): at least one iteration, stop once
                               ||alpha dx|| < tol, at most max_newton iterations, no status */
  skg_newton_record* record; /* host pointer, or NULL: skg_be_step fills it per Newton iteration */
  double ew_gamma;          /* pcg_rtol < 0: after the first Newton iteration the forcing term is
                               Eisenstat-Walker choice 2, ew_gamma (r_k / r_{k-1})^ew_alpha, raised to
                               ew_gamma eta_{k-1}^ew_alpha when that is above 0.1; 0 = 0.9 */
  double ew_alpha;          /* its exponent in [1, 2] (quarter steps are evaluated exactly alike on
                               the host and the device); 0 = 2 */
} skg_be_params;

typedef struct skg_be_state {
  double* u;                /* (3n) displacement from rest at the new step; in: ignored */
  const double* u_curr;     /* (3n) displacement at step k */
  const double* u_prev;     /* (3n) displacement at step k-1 */
  const double* mass;       /* (n) lumped vertex mass */
  const double* f_ext;      /* (3n) external force */
  const uint8_t* pinned;    /* (3n) 1 = DOF held at its rest position */
  const double* u_warm;     /* (3n) optional Newton initial guess (batched step): used per
                               instance only if the gradient norm there is below the one at
                               x_tilde; the relative residual stays judged against
                               ||g(x_tilde)|| */
  const double* u_prev2;    /* (3n) displacement at step k-2 (BDF2 only) */
  const double* u_prev3;    /* (3n) displacement at step k-3 (BDF2 only) */
  const double* x_rest;     /* (3n) rest positions (needed with contact planes) */
} skg_be_state;

typedef struct skg_step_info {
  int32_t newton_iters;
  int32_t pcg_iters;        /* summed over Newton iterations */
  int32_t ls_trials;        /* energy evaluations in line searches */
  int32_t status;           /* skg_status of the step */
  double residual0;         /* ||g(x_tilde)|| */
  double residual;          /* final ||g|| / residual0 */
  double min_alpha;         /* smallest accepted step */
  double energy;            /* final incremental potential relative to rest */
  int32_t launches;         /* kernels launched by the step */
  int32_t warm_used;        /* batched step: 1 if the warm start was kept, 0 if it fell back */
  double t_hessian_ms;      /* per-phase device time, filled when params->profile */
  double t_assemble_ms;
  double t_pcg_ms;
  double t_gradient_ms;
  double t_energy_ms;
} skg_step_info;

int64_t skg_be_workspace_size(const skg_tet_mesh* mesh, int precision);
/* One backward-Euler (or BDF2) step: Newton on the free DOFs from x_tilde = 2 x_k - x_{k-1}
 * with a PCG solve per iteration (block Jacobi, plus the coarse level when mesh->coarse
 * is attached) and Armijo backtracking, until the relative residual is below tol.
 * Host-synchronizes for its decisions. */
int skg_be_step(const skg_tet_mesh* mesh, const skg_be_params* params, const skg_be_state* state,
                void* workspace, skg_step_info* info_h, void* stream);

/* ---------------------------------------------------------------------- */
/* batched backward Euler: many independent meshes in one solve            */
/* ---------------------------------------------------------------------- */
/* The instances are concatenated into one skg_tet_mesh (disjoint vertex and tet
 * ranges, so its block pattern is block diagonal by instance).  Per instance,
 * Newton, the forcing term, the Armijo search and the convergence test are
 * those of skg_be_step; each instance's linear system is solved on a thread-block
 * cluster taken from a queue ordered largest first.  No counterpart call exists
 * in simkit (its user loops call backward_euler per mesh, backward_euler.py:27). */
typedef struct skg_batch {
  int32_t n_inst;
  int32_t max_rows;          /* block rows of the largest instance */
  const int32_t* inst_rows;  /* (n_inst+1) vertex (block-row) offsets */
  const int32_t* inst_tets;  /* (n_inst+1) tet offsets */
  const int32_t* vert_inst;  /* (n) instance of each vertex */
  const int32_t* tet_inst;   /* (t) instance of each tet */
  const int32_t* order;      /* (n_inst) instances by decreasing size */
} skg_batch;

int64_t skg_batch_workspace_size(const skg_tet_mesh* mesh, const skg_batch* batch, int precision);
/* One backward-Euler step of every instance; infos_h[n_inst] per instance, total_h summed.
 * An instance is converged when ||g|| < tol ||g(x_tilde)|| or, for instances that have come to
 * rest, ||g|| < 1e-10 ||f_ext|| (below that the relative test measures FP64 noise). */
int skg_be_step_batched(const skg_tet_mesh* mesh, const skg_batch* batch, const skg_be_params* params,
                        const skg_be_state* state, void* workspace, skg_step_info* infos_h, skg_step_info* total_h,
                        void* stream);

/* The same batched step with the Newton loop on the device, as a reusable plan.
 * skg_be_batch_plan_create records one call of skg_be_step_batched for these buffers into an
 * executable CUDA graph: every per-instance decision (relative-residual test, Eisenstat-Walker
 * forcing, Armijo trials, stop) is made by control kernels between the solver's kernels, and
 * the Newton iterations and line-search trials are conditional WHILE nodes those kernels drive
 * (the coarse refresh of the first iteration is a conditional IF node).  skg_be_batch_plan_step
 * launches the graph on `stream` and synchronizes once to return infos_h / total_h, the records
 * skg_be_step_batched returns.  The plan reads and writes through the pointers it was created
 * with (mesh and batch arrays, state buffers, workspace, the contents of *params and of the
 * contact planes): they must stay valid and their sizes unchanged until
 * skg_be_batch_plan_destroy; their contents may change between steps.  Uses no profiling
 * (params->profile is ignored) and allocates no device memory beyond the graph itself. */
typedef struct skg_batch_plan skg_batch_plan;
int skg_be_batch_plan_create(const skg_tet_mesh* mesh, const skg_batch* batch, const skg_be_params* params,
                             const skg_be_state* state, void* workspace, skg_batch_plan** plan_h);
int skg_be_batch_plan_step(skg_batch_plan* plan, skg_step_info* infos_h, skg_step_info* total_h, void* stream);
int skg_be_batch_plan_destroy(skg_batch_plan* plan);

/* skg_be_step with the Newton loop on the device: skg_be_plan_create records one call for these
 * buffers into an executable CUDA graph (the batch control kernels over one instance make the
 * decisions, the reductions are skg_be_step's own, the PCG takes its forcing term from device
 * memory); skg_be_plan_step launches it and synchronizes once to return the record skg_be_step
 * returns, for bitwise the same step (no phase times).  Same lifetime rules as the batch plan;
 * the plan allocates a few KB of device control state.  skg_be_plan_eligible returns 1 when the
 * parameters can be recorded: no profiling, no Newton record, stop_rule 0, and a PCG form that
 * runs as grid launches (the cluster form of small meshes and mode 0 need the host loop);
 * skg_be_plan_create returns SKG_ERR_ARG otherwise.  No counterpart in simkit, whose Newton loop
 * is host Python (solvers/newton.py:46-69). */
int skg_be_plan_eligible(const skg_tet_mesh* mesh, const skg_be_params* params);
int skg_be_plan_create(const skg_tet_mesh* mesh, const skg_be_params* params, const skg_be_state* state,
                       void* workspace, skg_batch_plan** plan_h);
int skg_be_plan_step(skg_batch_plan* plan, skg_step_info* info_h, void* stream);
int skg_be_plan_destroy(skg_batch_plan* plan);

/* ---------------------------------------------------------------------- */
/* generic sparse solve: replaces spsolve in newton_solver (newton.py:52)   */
/* ---------------------------------------------------------------------- */
/* Block-Jacobi PCG on a symmetric 3x3-block matrix in the layout above (FP64 values),
 * x = A^{-1} b to relative residual rtol. Workspace: skg_pcg_workspace_size. Writes
 * the iteration count to *iters_h (synchronizes). */
int64_t skg_pcg_workspace_size(int64_t n_rows_blocks);
int skg_pcg_bsr64(int64_t nbr, const int32_t* rowptr, const int32_t* col, const double* val, const double* b,
                  double* x, double rtol, int32_t max_iter, int32_t* iters_h, void* workspace, void* stream);

/* Allocation-free form of skg_pcg_bsr64 (no counterpart in the reference: simkit
 * calls scipy's spsolve, which allocates freely).  For callers that cannot call
 * cudaMalloc while they solve - a real-time simulation loop that must not stall
 * on an allocation, or a host program that owns every device buffer and passes
 * only inputs and outputs.  Its scratch is one fixed device array inside the
 * library (about 1 MB, held by every GPU that loads the library until exit),
 * enough for at most skg_pcg_noalloc_max_rows() block rows (4096, i.e. 12,288
 * unknowns); larger systems return SKG_ERR_CAPACITY.  Every call looks up the
 * array's device address on the current device (cudaGetSymbolAddress); the first
 * call on a device also loads the library there and should come before any
 * stream capture.  Each call synchronizes `stream` to read the solve's status.
 * All calls share that array, so calls that overlap on the GPU race; serialise
 * them.  Allocates no device memory. */
int64_t skg_pcg_noalloc_max_rows(void);
int skg_pcg_bsr64_noalloc(int64_t nbr, const int32_t* rowptr, const int32_t* col, const double* val,
                          const double* b, double* x, double rtol, int32_t max_iter, int32_t* iters_h,
                          void* stream);

/* Self-test of the bounded device waits (no counterpart in the reference, which
 * has no device code).  kind 0 runs the grid barrier of the grid-persistent PCG
 * forms with one of its two blocks never arriving; kind 1 runs the mbarrier wait
 * of the cluster PCG's bulk-copy pipeline on a phase that never completes.  The
 * wait gives up after `limit` polls (1..2^24; the solvers use 2^24 for the grid
 * barrier and 2^20 for the mbarrier) and *status_h receives SKG_ERR_TIMEOUT, the
 * status the solvers return when a wait gives up; the context stays usable.
 * Workspace: skg_wait_selftest_workspace_size() bytes.  Synchronizes `stream`. */
int64_t skg_wait_selftest_workspace_size(void);
int skg_wait_selftest(int kind, int64_t limit, int32_t* status_h, void* workspace, void* stream);

/* ---------------------------------------------------------------------- */
/* learned warm start: BF16 tensor-core MLP pieces (no simkit counterpart)  */
/* ---------------------------------------------------------------------- */
/* C[R x Nc] = A[R x L] B[Nc x L]^T on the 5th-generation tensor cores (tcgen05, TMEM
 * accumulators, TMA-loaded 128-byte-swizzled tiles).  A, B BF16 (row pitches lda, ldb
 * elements, 16-byte aligned), L a multiple of 64, Nc a multiple of 16 <= 256.
 * epi 0: FP32 out_f32 (+bias), per split [splits][R][ld_out]; 1: z = acc + bias ->
 * out_z (bf16), gelu(z) -> out_h (bf16); 2: bf16 out_h (+bias).  err: device int set
 * to SKG_ERR_TIMEOUT if a bounded wait gave up. */
int skg_mlp_gemm(const void* A, int64_t R, int64_t lda, const void* B, int Nc, int64_t ldb, int64_t L, int splits,
                 int epi, const float* bias, float* out_f32, void* out_z, void* out_h, int Nstore, int ld_out,
                 int* err, void* stream);
/* dZ = dH * gelu'(Z) elementwise (BF16). */
int skg_mlp_gelu_backward(const void* dH, const void* Z, int64_t n, void* dZ, void* stream);
/* out = in^T for a rows x cols BF16 matrix. */
int skg_mlp_transpose(const void* in, int rows, int cols, int ld_in, void* out, int ld_out, void* stream);
/* out = sum over splits of part[s] (fixed order). */
int skg_mlp_reduce_splits(const float* part, int splits, int64_t n, float* out, void* stream);
/* db[c] = sum over rows of dZ[r][c] (fixed order). */
int skg_mlp_colsum(const void* dZ, int rows, int cols, int ld, float* db, void* stream);
/* mean squared error of y against t and its gradient dy (BF16); scratch: 2051 doubles. */
int skg_mlp_mse(const float* y, int ld_y, const float* t, int rows, int cols, void* dy, int ld_dy, double* scratch,
                double* loss_h, void* stream);
/* one Adam step on FP32 weights; refreshes a BF16 copy and optionally its transpose. */
int skg_mlp_adam(float* w, const float* grad, float* m1, float* m2, int rows, int cols, float lr, float b1, float b2,
                 float eps, int step, void* w16, int ld16, void* wt16, int ldt, void* stream);

/* MLP input rows [n][64] BF16 for one frame: per-vertex features (rest position,
 * displacement, last-step velocity and Newton correction in units of 9.8 dt^2,
 * gravity) and a 32-value per-instance mean-pooled context.  vf (n x 16 f32) and
 * ctx (n_inst x 32 f32) are caller scratch; corr may be null. */
int skg_warmstart_features(const double* X, const double* u, const double* u_prev, const double* corr,
                           const double* f_ext, const double* mass, double dt, int64_t n, const int32_t* inst_rows,
                           const int32_t* vert_inst, int n_inst, const float* inst_scalars, float* vf, float* ctx,
                           void* out, void* stream);
/* u_warm = u_tilde + corr + 9.8 dt^2 * pred[:, 0:3] (pinned DOFs stay at u_tilde): the network
 * refines the second-order extrapolation u_tilde + corr, corr = the previous step's Newton
 * correction; corr and pred may be null. */
int skg_warmstart_apply(const double* u_tilde, const double* corr, const float* pred, int ld_pred,
                        const uint8_t* pinned, double dt, int64_t n, double* u_warm, void* stream);
/* training targets (u_next - u_tilde - corr) / (9.8 dt^2), [n][3] FP32 (corr may be null). */
int skg_warmstart_targets(const double* u_next, const double* u_tilde, const double* corr, double dt, int64_t n,
                          float* t, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SIMKIT_GB300_H_ */
