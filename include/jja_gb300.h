/*
 * jja_gb300.h — C ABI of the GB300 (sm_103a) RCSJ time-stepping library libjja_gb300.so.
 *
 * The reference (pyjjasim) has no native layer: its hot path is the Python function
 * time_evolution_core(problem, th_store_mask, I_store_mask) (time_evolution.py:461-582),
 * called by time_evolution() (:443) from TimeEvolutionProblem.compute() (:303-307).
 * These entry points replace the pieces of that function; the ctypes binding in
 * pyjjasim_gb300/_native.py calls them.
 *
 * Conventions: plain pointers and sizes, no framework types. Functions return 0 on success
 * and a nonzero jja_status otherwise; jja_last_error() gives the message (per thread).
 * "device" pointers are CUDA global-memory pointers on the current device; "host" pointers
 * are ordinary memory. Arrays indexed (j, w) are row-major with the problem index w
 * contiguous: element (j, w) is at j*W + w (the reference's (Nj, W) layout).
 */
#ifndef JJA_GB300_H
#define JJA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  JJA_OK = 0,
  JJA_ERR_ARG = 1,        /* invalid argument / shape */
  JJA_ERR_NOT_SPD = 2,    /* face-space matrix is not positive definite */
  JJA_ERR_CUDA = 3,       /* a CUDA runtime call failed */
  JJA_ERR_NONFINITE = 4,  /* a time step produced a NaN or +-inf phase (reported by jja_plan_check) */
  JJA_ERR_INTERNAL = 5
} jja_status;

typedef struct jja_factor jja_factor;
typedef struct jja_plan jja_plan;

/* ---------------------------------------------------------------- host factorisation --- */

typedef struct {
  int nd_leaf;        /* nested-dissection leaf size (<= 0: default 8) */
  int max_supernode;  /* cap on supernode width (0: none) */
  int keep_factor;    /* keep plain Cholesky columns for host checks */
  int relax_zeros;    /* merge a child supernode into its parent if that adds <= this many zeros */
  double relax_frac;  /* ... or <= this fraction of the merged block (both 0: fundamental only;
                         negative values select the defaults 16 and 0.05) */
} jja_factor_opts;

typedef struct {
  int n;              /* matrix order (faces) */
  int n_supernodes;
  int n_levels;       /* levels of the supernodal elimination tree */
  int max_k, max_m;   /* widest supernode, longest off-diagonal row list */
  int64_t nnz_L;      /* nonzeros of L (supernodal, lower triangle incl. diagonal) */
  int64_t f_values;   /* doubles in the (k+m) x k solve blocks */
  double factor_flops;
} jja_factor_stats;

/* Orders and factorises the face-space matrix K = A (L + diag(1/c0)) A^T
 * (time_evolution.py:504-506, where the reference calls scipy.sparse.linalg.factorized).
 * K: n x n symmetric, full pattern (both triangles), CSC with 64-bit column pointers.
 * coord_x/y: optional face coordinates (centroids) that seed the nested dissection; NULL to
 * derive coordinates from breadth-first distances. perm: optional fill-reducing order
 * (new -> old) that replaces the nested dissection. Runs on the host; no GPU needed. */
int jja_factor_create(int n, const int64_t* colptr, const int32_t* rowind, const double* val,
                      const double* coord_x, const double* coord_y, const int32_t* perm,
                      const jja_factor_opts* opts, jja_factor** out);
void jja_factor_destroy(jja_factor* f);
int jja_factor_get_stats(const jja_factor* f, jja_factor_stats* out);
/* perm_out[n]: new -> old face order used by the factor (a postordered nested dissection). */
int jja_factor_get_perm(const jja_factor* f, int32_t* perm_out);
/* Supernode table (arrays of n_supernodes entries, any may be NULL): first column, width k,
 * off-diagonal row count m, elimination-tree level (leaves 0) and parent (-1 at roots). */
int jja_factor_get_supernodes(const jja_factor* f, int32_t* col0, int32_t* k, int32_t* m, int32_t* level,
                              int32_t* parent);
/* Host solve K x = b in place (b: n x nrhs row-major, original order). Diagnostic only:
 * used to check a factor without a GPU; the time-stepping path solves on the GPU. */
int jja_factor_solve_host(const jja_factor* f, double* b, int nrhs);

/* ------------------------------------------------------------------------ GPU plan --- */

/* Launch shape of the triangular-solve kernels; 0 in a field selects its default. The
 * project's autotuner (pyjjasim_gb300/autotune.py) times candidates and picks these. */
typedef struct {
  int rhs_block;      /* problems per warp: a power of two <= 32 (default min(W, 32) rounded up) */
  int rows_per_lane;  /* output rows per lane of a work item: 1, 2, 4 or 8 (default 1) */
  int target_warps;   /* levels with fewer work items split their dot products until they have
                         this many (default 152 x 24; 152 x 64 for 2-16 problems) */
  int min_piece;      /* shortest piece of a split dot product (default 16) */
  int schedule;       /* 1: one launch per elimination-tree level; 2: dataflow, one persistent
                         launch per sweep whose work items wait (bounded) on per-supernode
                         completion counters; 3: cooperative, one launch per sweep that walks the
                         levels separated by bounded grid-wide barriers; 0: default (1) */
  int rows_per_lane_fwd; /* rows per lane of the forward sweep alone (0: rows_per_lane if set,
                            else the forward default: 2 for W >= 256 and for W >= 8 on 2^17 faces
                            or more, 1 otherwise) */
  int pack_rows;      /* W = 1, level schedule: supernodes of at most this many rows (and at most 8
                         columns) are solved one per lane, 32 per warp (0: default 24; negative:
                         never) ... */
  int pack_min_warps; /* ... on levels whose regular items need at least this many warps
                         (0: default 4864, half a wave of 152 SMs x 64 warps) */
  int pdl;            /* 1: launch the step's kernels with programmatic dependent launch (each
                         launch overlaps the tail of the kernel before; measured: 6 % faster for
                         W = 1, 5-7 % slower for W >= 64); 0: default (plain launches) */
  int groups;         /* level schedule: step the problems as this many independent groups, each
                         on its own stream (created by the plan; the call's stream forks to them
                         and joins back before jja_run returns), so their launch chains overlap;
                         0: default (W / 160 clamped to [2, 4] from W = 256 on, else 1) */
  int coop_blocks;    /* cooperative schedule: at most this many blocks per sweep launch (0: two per
                         SM, fewer when the widest level has fewer work items) */
  int dst_lines;      /* fast Poisson solve (jja_plan_set_fast_poisson): grid lines per block of the
                         sine-transform kernels, 1 or 2 (two real lines share one complex FFT);
                         0: default (2 when that still gives at least 2 x 152 blocks, else 1) */
  int pack_lanes;     /* W = 1 packs: lanes per packed supernode, 1, 2 or 4 (its rows split between
                         them; 32 / pack_lanes supernodes per warp); 0: default (per level: 4 where
                         one lane per supernode would give fewer than 4096 warps, else 1) */
  int subtree_rows;   /* level schedule: subtrees at the bottom of the elimination tree spanning at
                         most this many rows (their columns plus their root's off-diagonal rows,
                         <= 64) are solved in shared memory in one launch per sweep, before the
                         levels above them: from 32 problems per warp (W >= 17) one warp per subtree
                         and 32 problems; below that 32 / WB subtrees of one shape per warp, WB
                         problems each (W = 1: 32 subtrees, one per lane). 0: default (32 rows, 16
                         at W = 1; at W >= 17 where the launch has at least 152 x 16 warps, below
                         where the packs fill at least 152 x 4 warps; measured 5-8 % per step at
                         W = 512-1024 on 128x128 arrays and at W = 8 on 1024x1024, 4-8 % on W = 1
                         ragged unions); negative: never */
} jja_solve_tuning;

/* Builds on the host (no GPU needed) the work-item schedule that jja_plan_create would make for
 * W problems with `tuning` (NULL: defaults) and checks the dataflow order: every item waits only
 * for items before it in its sweep, on counts equal to the items that will count. Returns
 * JJA_ERR_INTERNAL when that fails (jja_plan_create makes the same check); the item counts of
 * the two sweeps go to n_fwd_items / n_bwd_items (either may be NULL). */
int jja_factor_check_schedule(const jja_factor* f, int W, const jja_solve_tuning* tuning, int64_t* n_fwd_items,
                              int64_t* n_bwd_items);

/* Shape of that schedule (host only, no GPU needed). */
typedef struct {
  int n_levels;            /* level launches per sweep (above the subtrees) */
  int n_subtrees;          /* bottom subtrees solved in shared memory (0: none) */
  int n_subtree_members;   /* supernodes inside them (they have no level items) */
  int max_subtree_rows;    /* largest subtree: columns plus its root's off-diagonal rows */
  int n_pack_items;        /* below 32 problems per warp: warps of subtree packs */
  int n_pack_shapes;       /* ... distinct subtree shapes among them */
  int64_t n_fwd_items;     /* level work items of the forward sweep */
  int64_t n_bwd_items;     /* ... of the backward sweep */
} jja_schedule_stats;
int jja_factor_schedule_stats(const jja_factor* f, int W, const jja_solve_tuning* tuning, jja_schedule_stats* out);

typedef struct {
  int Nj, Nf, W;           /* junctions, faces, problems per launch */
  int stencil_width;       /* 3, 4 or 5 (time_evolution.py:401-408) */
  /* cycle matrix A (Nf x Nj, entries +-1) as CSR over the original face order */
  const int64_t* a_rowptr; /* Nf+1 */
  const int32_t* a_col;    /* junction index */
  const double* a_val;     /* +1 / -1 */
  /* per-junction coefficients (host arrays of length Nj) */
  const double* Ic;        /* critical current (DefaultCPR: Ic sin(theta)) */
  const double* inv_c0;    /* 1 / c0, c0 = s1[0] Rv + s2[0] Cv (time_evolution.py:477) */
  const double* coef;      /* (stencil_width-1) x Nj: c_k = s1[k] Rv + s2[k] Cv, k = 1.. */
  const double* Rv;        /* 1 / (dt R), noise amplitude sqrt(2 T Rv) (time_evolution.py:537) */
  double extrap[4];        /* CPR argument weights on theta(t-1), theta(t-2), ... (:547-553) */
  double dt;
  const double* Ic_w;      /* optional (Nj x W) critical currents per problem (replaces Ic): W
                              disorder realisations share one face-space matrix, since K does not
                              depend on Ic; NULL to use Ic for every problem */
  jja_solve_tuning tuning; /* all zero: defaults */
} jja_plan_desc;

/* Uploads the circuit tables and the factor to the current CUDA device and allocates the
 * face-space work vectors for W problems (cudaMalloc). The factor may be destroyed after. */
int jja_plan_create(const jja_plan_desc* desc, const jja_factor* f, jja_plan** out);
void jja_plan_destroy(jja_plan* p);
/* Bytes of device memory held by the plan (tables + factor + work vectors). */
int64_t jja_plan_device_bytes(const jja_plan* p);
/* Fast Poisson solve of uniform square arrays (the row SquareArray reserves for it,
 * josephson_circuit.py:958 `_Asq_dst_K`): when K = kappa (4 I - adjacency) on an mx x my grid of
 * faces (equal R and C, a uniform self-inductance; K = kappa times the 5-point Dirichlet
 * Laplacian), every face-space solve of the plan (time steps, jja_solve, the adjoint) becomes
 * three sine-transform kernels instead of the triangular sweeps. grid_face[iy * mx + ix] (host,
 * mx * my entries): the face (original order) at grid cell (ix, iy); mx + 1 and my + 1 powers of
 * two up to 1024. The caller checks that K has that form. jja_solve_static keeps the sweeps. */
int jja_plan_set_fast_poisson(jja_plan* p, int mx, int my, const int32_t* grid_face, double kappa);
/* Synchronises the device, then reads and clears the plan's device error flags: *flow_timeouts
 * = 1 if a wait of a dataflow sweep ran out of its bound since the last call (the results of
 * those steps are invalid), else 0. Returns JJA_ERR_NONFINITE when a time step of jja_run /
 * jja_run_timed produced a NaN or +-inf phase since the last call (a diverging run: NaN or inf
 * in an input, or a time step too large for the circuit); the state is then invalid. */
int jja_plan_check(jja_plan* p, int* flow_timeouts);
/* Test of the bounded waits: runs one forward dataflow sweep whose wait counts can never be
 * reached (a plan of the cooperative schedule: one cooperative sweep whose grid barriers wait for
 * one block more than the launch has), then synchronises `stream`. Every wait gives up (the
 * first after its bound, the rest at once), the kernel returns, and the plan's error flag is set
 * for jja_plan_check to report. The plan's face-space work vectors hold garbage afterwards; the
 * plan stays usable. */
int jja_plan_test_wait_limit(jja_plan* p, void* stream);

/* A source on the device: at step i, value(n, w) = ptr[n*stride_n + w*stride_w + (i - t0)*stride_t]
 * (element strides; 0 broadcasts). stride_t == 0: the same value at every step. stride_t != 0:
 * a window of time steps [t0, t0 + steps) held on the device (t0 and steps are jja_state.src_t0
 * and src_steps), which replaces the reference's per-step evaluation of time-dependent inputs
 * (time_evolution.py:334-340, 523-531). ptr == NULL means the source is identically zero. */
typedef struct {
  const double* ptr;
  int64_t stride_n;
  int64_t stride_w;
  int64_t stride_t;
} jja_view;

enum { JJA_NOISE_NONE = 0, JJA_NOISE_BUFFER = 1, JJA_NOISE_PHILOX = 2 };

typedef struct {
  double* hist[4];       /* device (Nj x W): theta at t-1, t-2, ... (stencil_width-1 used);
                            jja_run rotates them: on return hist[0] is the newest phase */
  double* theta_s;       /* device (Nj x W) accumulated voltage-source phase, or NULL */
  jja_view Is;           /* current sources (Nj rows) */
  jja_view f;            /* external flux (Nf rows, original face order) */
  jja_view Vs;           /* voltage sources (Nj rows) */
  jja_view T;            /* temperature (Nj rows) */
  int noise_mode;        /* JJA_NOISE_* */
  const double* noise;   /* JJA_NOISE_BUFFER: device (Nj x W) standard normals of this step */
  uint64_t seed;         /* JJA_NOISE_PHILOX: key */
  int64_t step;          /* index of the first step of the call (Philox counter) */
  double* th_out;        /* device (slots x Nj x W) or NULL */
  double* I_out;         /* device (slots x Nj x W) or NULL */
  int64_t src_t0;        /* first step held by the time-dependent views (stride_t != 0) */
  int64_t src_steps;     /* steps they hold: a call must satisfy src_t0 <= step and
                            step + nsteps <= src_t0 + src_steps */
  int store_all;         /* 1: step i of a jja_run call is stored in slot i of th_out / I_out
                            (th_slot / I_slot must be NULL); such runs replay CUDA graphs too */
} jja_state;

/* Runs nsteps time steps of the RCSJ update (time_evolution.py:523-580) on `stream`
 * (a cudaStream_t, NULL = default stream). th_slot[i] / I_slot[i] (host arrays of length
 * nsteps, or NULL) give the output slot of step i or -1. With use_graph != 0 runs of steps
 * that store nothing are captured into CUDA graphs (a few are cached per plan, keyed by the
 * state's buffers) and replayed. */
int jja_run(jja_plan* p, jja_state* st, int nsteps, const int64_t* th_slot, const int64_t* I_slot,
            int use_graph, void* stream);

/* Like jja_run (no stored outputs, no graph) but records CUDA events at the stage boundaries
 * of every step. stage_ms[6] receives the summed device time of: junction currents,
 * face right-hand side, forward solve, backward solve, update; and [5] the whole run. With
 * problem groups every stage runs the groups concurrently and joins them before its closing
 * event (the stages do not overlap each other, as they do in jja_run). Used by the benchmark
 * to attribute step time to kernels; same results as jja_run. */
int jja_run_timed(jja_plan* p, jja_state* st, int nsteps, double* stage_ms, void* stream);

/* ---------------------------------------------------------------------------- adjoint --- */
/* No counterpart in the reference (which has no derivatives): backward-through-time steps of
 * the width-3 update for gradients of a loss L = sum_n <G_n, theta_n>. With a_n = dL/dtheta_n
 * and mu_n = Q a_n, Q = D A^T K^-1 A D - D (D = diag(1/c0)), one call computes, for step n,
 *   a_n   = G_n + (2 Ic cos phi_{n+1} + c1) mu_{n+1} + (-Ic cos phi_{n+2} + c2) mu_{n+2}
 *   mu_n  = Q a_n  (one face-space solve with the same factor; K is symmetric)
 * and accumulates usum += D a_n, musum += mu_n, gIc += mu_n sin phi_n, phi_n = 2 th_{n-1} - th_{n-2}.
 * Then dL/dIc = gIc, dL/dIs = -musum, dL/df = -2 pi K^-1 A usum (jja_adjoint_flux).
 * All arrays are device (Nj x W) except G (a view, NULL ptr = 0). */
typedef struct {
  jja_view G;             /* direct loss weights at step n (Nj rows) */
  const double* th_m1;    /* theta_{n-1} */
  const double* th_m2;    /* theta_{n-2} */
  const double* mu_p1;    /* mu_{n+1}, NULL past the last step */
  const double* mu_p2;    /* mu_{n+2}, NULL past the last step */
  const double* cos_p1;   /* cos(phi_{n+1}) written by the call for step n+1 */
  const double* cos_p2;   /* cos(phi_{n+2}) */
  double* mu_out;         /* mu_n */
  double* cos_out;        /* cos(phi_n) */
  double* usum;           /* accumulators, zero before the first (last-step) call */
  double* musum;
  double* gIc;
} jja_adjoint_args;

int jja_adjoint_step(jja_plan* p, const jja_adjoint_args* args, void* stream);

/* The adjoint steps of one recomputed segment, from its last step down to its first (the loop
 * of jja_adjoint_step calls without a host round trip per step). */
typedef struct {
  const double* seg;       /* device (L + 2) x Nj x W: theta_{s0-2}, theta_{s0-1}, theta_{s0}, ..., theta_{s0+L-1} */
  int64_t s0, L, Nt;       /* first step of the segment, its length, steps of the whole run */
  const double* const* G;  /* host array of L device pointers (Nj x W loss weights of step s0 + i) or
                              NULL entries / NULL array where a step has none */
  double* mu[3];           /* device (Nj x W) ring buffers of mu, indexed by step % 3 */
  double* cos[3];          /* device (Nj x W) ring buffers of cos(phi), indexed by step % 3 */
  double* usum;            /* accumulators as in jja_adjoint_args */
  double* musum;
  double* gIc;
  int use_graph;           /* 1 (non-default stream): capture the walk once per distinct set of
                              buffers, step % 3 phase and loss-weight pointers, then replay it */
} jja_adjoint_segment_args;

int jja_adjoint_segment(jja_plan* p, const jja_adjoint_segment_args* args, void* stream);
/* gf (device Nf x W, original face order) = -2 pi K^{-1} A usum: the flux gradient. */
int jja_adjoint_flux(jja_plan* p, const double* usum, double* gf, void* stream);

/* Face-space solve on the device: x = K^{-1} b for W right-hand sides (device arrays
 * Nf x W, original face order). Exposed for tests of the triangular-solve kernels. */
int jja_solve(jja_plan* p, const double* b, double* x, void* stream);

/* Allocation-free variant of jja_solve. No counterpart in the reference: it exists for callers
 * that cannot allocate device memory when they solve — code running after all device memory has
 * been handed to another allocator (a framework's caching pool) or under a hard memory budget,
 * and per-step loops that must not pay the device-wide synchronisation of cudaMalloc/cudaFree.
 * It uses the plan's factor tables and, instead of the plan's work vectors, a fixed 32 MiB
 * device array inside the library (held by every GPU that loads the library until exit); it
 * calls no cudaMalloc, cudaFree or allocating library routine. Limit: 2 x Nf x W doubles must fit,
 * i.e. Nf * W <= 2,097,152 (for example a 128 x 128 array with W <= 130); larger plans get
 * JJA_ERR_ARG with the limit in the message. The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress), so make that first call before any stream capture.
 * The address is looked up again when the device's context was destroyed and created again
 * (cudaDeviceReset); that call, too, must come before any stream capture.
 * All calls share the array: calls that overlap on the GPU (different streams or threads) race.
 * b and x are caller-owned device arrays (Nf x W, original face order), as for jja_solve. With a
 * plan of the dataflow schedule (tuning.schedule = 2) a sweep's bounded wait can run out: the call
 * still returns 0, so synchronise and call jja_plan_check to confirm the result is valid. */
int jja_solve_static(jja_plan* p, const double* b, double* x, void* stream);

/* -------------------------------------------------------------------- static problems --- */
/* The reference's static (stationary) problem solver on the GPU: the Newton iteration
 * static_compute (static_problem.py:1400-1515) and the London approximation
 * london_approximation (:1378-1395), for W problems on one circuit at once. Every Newton
 * iteration refactors A (L + diag(1/q)) A^T, q = Ic cos(theta), numerically on the device
 * (supernodal LDL^T on the symbolic structure of `factor`, which must have the sparsity pattern
 * of A (L + D) A^T for a diagonal D, e.g. the factor of A (L + I) A^T), and solves with it.
 * Vectors are problem-major device arrays: (W x Nj) per junction, (W x Nf) per face (original
 * face order), element (w, j) at w*Nj + j. */
typedef struct jja_static jja_static;

typedef struct {
  int Nj, Nf, Nn, W;          /* junctions, faces, nodes, problems */
  const int64_t* a_rowptr;    /* cycle matrix A (Nf x Nj, entries +-1), CSR over the original face order */
  const int32_t* a_col;
  const double* a_val;
  const int64_t* m_rowptr;    /* cut matrix M (Nn x Nj), CSR (Kirchhoff residual) */
  const int32_t* m_col;
  const double* m_val;
  const int64_t* l_rowptr;    /* inductance L (Nj x Nj), CSR; all NULL when the circuit has none */
  const int32_t* l_col;
  const double* l_val;
  const int64_t* kl_colptr;   /* A L A^T (Nf x Nf, both triangles, CSC over the original face order); NULL: none */
  const int32_t* kl_rowind;
  const double* kl_val;
  const double* Ic;           /* critical currents (Nj) */
  double A_norm, M_norm;      /* ||A||_2 and ||M||_2 (sqrt of the largest eigenvalue of A A^T, M M^T),
                                 the normalisers of the reference's residuals (josephson_circuit.py:762-780) */
} jja_static_desc;

int jja_static_create(const jja_static_desc* desc, const jja_factor* factor, jja_static** out);
void jja_static_destroy(jja_static* sp);
int64_t jja_static_device_bytes(const jja_static* sp);

/* Diagnostic of the device factorisation: x_w = (A (L + diag(iq_w)) A^T)^-1 b_w for every problem
 * (iq: device W x Nj, b, x: device W x Nf). pivot_errors (host, W entries, or NULL) receives 1 for a
 * problem whose elimination met a zero or non-finite pivot (the matrix may be indefinite; the
 * elimination does not pivot). */
int jja_static_solve(jja_static* sp, const double* iq, const double* b, double* x, int* pivot_errors, void* stream);

/* London approximation in phase zone n (static_problem.py:1378-1395):
 * theta = iIc (A^T (A (iIc + L) A^T)^-1 (2 pi (n - f) - A (iIc + L) Is) + Is), iIc = 1/Ic (0 where
 * |Ic| <= 1e-12). Is, theta: device W x Nj; f: device W x Nf; n: device W x Nf int32. */
int jja_static_london(jja_static* sp, const double* Is, const double* f, const int32_t* n, double* theta,
                      void* stream);

typedef struct {
  double* theta;              /* device W x Nj: initial guess in, solution out */
  const double* Is;           /* device W x Nj current sources */
  const double* f;            /* device W x Nf external flux (phase zone z = 0, as StaticProblem.compute uses) */
  const int32_t* n;           /* device W x Nf target vortex configuration */
  double tol;                 /* residual tolerance (the reference's default 1e-10) */
  int maxiter;                /* iteration limit (default 30) */
  int stop_as_residual_increases;   /* stop when error(iter) > error(iter - 3) (default 1) */
  int stop_if_not_target_n;         /* the reference's flag, with its behaviour (default 0) */
} jja_newton_args;

typedef struct {               /* host arrays the caller provides */
  int* status;                /* W: 0 converged on the target configuration, 1 diverged, +2 at maxiter */
  int* iterations;            /* W: Newton steps taken */
  double* residuals;          /* W x (maxiter + 1): max(Kirchhoff, winding) residual per iterate (0 past the last) */
  int* is_target;             /* W x (maxiter + 1): 1 where the iterate has the target vortex configuration */
} jja_newton_result;

/* static_compute for every problem: the stop rules, residuals and status of the reference's
 * Newton iteration (static_problem.py:1476-1515, NewtonIterInfo :88-201); every problem stops on
 * its own. The reference's NaN rule is kept (theta += 1e10 when the solve is not finite). */
int jja_static_newton(jja_static* sp, const jja_newton_args* args, jja_newton_result* result, void* stream);

/* Vortex configurations of n_steps stored phase arrays theta (device, n_steps x Nj x W):
 * n_s(f, w) = -sum_j A_fj round(theta_s(j, w) / 2 pi) (TimeEvolutionResult.get_vortex_configuration,
 * time_evolution.py:734-755), written to n_out (device n_steps x Nf x W int32, original face
 * order) when not NULL; and flow[w] += sum_f sum_{s>=1} |n_s(f,w) - n_{s-1}(f,w)| (device W
 * uint64; the numerator of AnnealingProblem's vortex mobility, :1131-1136) when not NULL. */
int jja_vortex(jja_plan* p, const double* theta, int64_t n_steps, int32_t* n_out, uint64_t* flow, void* stream);

/* out[i] = sin(x[i]) with the library's device sine (device arrays of n doubles), the one
 * the junction-current kernels use for Ic sin(theta) (pyjjasim static_problem.py:82-85): 64-bit
 * fixed point and FP32, no FP64 instruction; within 1.2e-16 of a correctly rounded sine for
 * |x| < 2^62, NaN from 2^62 on. Exposed so tests can bound its error. */
int jja_eval_sin(jja_plan* p, const double* x, double* out, int64_t n, void* stream);

/* The same sine (and the cosine the adjoint uses) evaluated on the host by the same source code
 * (64-bit fixed point and FP32, no GPU needed): s[i] = sin(x[i]), c[i] = cos(x[i]) for host
 * arrays of n doubles; either output may be NULL. A diagnostic: tests check the algorithm's
 * error on the CPU over many more points than a GPU run needs. */
int jja_sin_host(const double* x, double* s, double* c, int64_t n);

/* Message of the last failing call on this thread ("" if none). */
const char* jja_last_error(void);
/* Number of kernel launches the library issued since load (for launch accounting). */
int64_t jja_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif /* JJA_GB300_H */
