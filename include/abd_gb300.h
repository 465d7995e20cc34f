/*
 * abd_gb300 — C ABI of the GB300 affine-body contact step.
 *
 * One handle owns one (possibly batched) scene resident in GPU memory and advances it
 * one frame at a time with the reference's per-frame step (ABD::implicit_euler,
 * model/abd.cpp:30-140): iAABB culling into point-triangle / edge-edge / vertex-ground
 * pair sets, IPC barrier + lagged friction terms projected to PSD, the 12x12
 * block-sparse Newton system, a block-Jacobi PCG solve, the CCD step bound and the
 * Armijo line search. Every call returns an abd_status; nothing exits the process.
 *
 * Plain pointers and sizes only; all host arrays are owned by the caller and copied.
 * One thread per handle; handles are independent. Body state layout per body:
 * 12 doubles q = [p(3), a1(3), a2(3), a3(3)], a_k the columns of A (x = A xbar + p),
 * the same order as the reference's `cat(c.q)` (model/mutils.cpp:44-51) and its trace
 * files (player_save, model/mutils.cpp:293-329).
 */
#ifndef ABD_GB300_H
#define ABD_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  ABD_OK = 0,
  ABD_ERR_NAN = 1,            /* non-finite Newton step (reference: exit(1), abd.cpp:288-291) */
  ABD_ERR_LS_STALL = 2,       /* line search hit its trial cap (reference: unbounded loop) */
  ABD_ERR_PAIR_OVERFLOW = 3,  /* a pair buffer could not be grown */
  ABD_ERR_TOI_TINY = 4,       /* TOI < 1e-6 twice in a row (reference: exit(1), iaabb.cpp:306-313) */
  ABD_ERR_NOT_SPD = 5,        /* a diagonal block was not positive definite */
  ABD_ERR_PCG_NOCONV = 6,     /* PCG hit its iteration cap (the step is still taken) */
  ABD_ERR_CUDA = 7,           /* CUDA runtime error; see abd_last_error */
  ABD_ERR_INVALID = 8,        /* invalid argument */
  ABD_ERR_IO = 9,             /* config / scene / mesh file could not be read */
  ABD_ERR_SAME_DIRECTION = 10 /* Newton step repeats the previous one (abd.cpp:181-188) */
} abd_status;

/* Step parameters. Field names follow the reference's config.json keys
 * (view/control.cpp:19-111); dhat, ortho_kappa and ground_offset are the values the
 * reference hard-codes (barrier.cpp:7-8, othogonal_energy.cpp:8, geometry.cpp:60). */
typedef struct {
  double dt;
  double kappa;          /* barrier stiffness ("kappa") */
  double dhat;           /* squared-distance activation distance */
  double ortho_kappa;    /* orthogonality stiffness */
  double ground_offset;  /* vertex-ground distance is y + ground_offset (0.5) */
  double mu;             /* friction coefficient */
  double evh;            /* friction epsilon_v * h = dt * evh */
  double eps_x;          /* edge-edge mollifier scale */
  double backoff;        /* CCD backoff factor */
  double c1;             /* Armijo constant (params_double.c1) */
  double tol;            /* Newton tolerance on |dq| (params_double.tol) */
  double max_uk;         /* params_double.max_uk */
  double gravity_y;      /* -9.8 with "gravity": true */
  double ls_grad_tol;    /* line search stops when |grad| <= this (1e-3 in the reference) */
  double pcg_rel_tol;    /* PCG relative residual target */
  int max_iter;          /* cumulative Newton cap, as the reference's `iter` member */
  int ground, pt, ee, psd, line_search, upper_bound;
  int vg_fric, pt_fric, ee_fric, clip;
  int pcg_max_iter;
  /* broad-phase selection (view/control.cpp:37-68): iaabb odd culls with iAABB, even with
   * the spatial hash; iaabb > 1 bounds the step with the iAABB trajectory pass, otherwise
   * with step_size_upper_bound (hashed trajectories when full_ccd, else the d_sqrt bound) */
  int iaabb, full_ccd;
  double safe_factor;    /* spatial-hash distance scale */
  double sh_min_xyz, sh_dx; /* "spatial hashing": cell = int(max(x - min_xyz, 0) / dx) */
  int sh_xyz_bits;       /* bucket = low xyz_bits bits of each cell coordinate */
  int sh_fix_edge_trajectory; /* 1: register edge trajectories by both ends (the reference
                                 registers them by their start, upper_bound.cpp:151) */
  double dq_tol;         /* params_double.dq_tol: same-direction stop (abd.cpp:181-188) */
  int damping;           /* "damping": {"enable"}: H (1 + beta) + diag(m, Ic) (alpha - beta)
                            (damping_sparse, mutils.cpp:106-115) */
  double damp_alpha, damp_beta;
  /* Newton solve (the reference factorizes directly, abd.cpp:229-303): after the PCG,
   * pcg_refine passes of iterative refinement, each solving H d = b - H x with the true
   * residual to pcg_refine_tol relative and adding d, bring the solution to the backward
   * error of a direct solve. */
  int pcg_refine;
  double pcg_refine_tol;
  /* "solver" (view/control.cpp:29-30): 0 "sparse" (block-Jacobi PCG over the block-sparse
   * system), 1 "dense" (the scene's full 12 n x 12 n matrix factorized by a dense Cholesky,
   * as the reference's big_hess.ldlt(), abd.cpp:233-264; for small scenes) */
  int solver;
  /* Newton iterations per frame at most, per scene (0: unbounded, as the reference's loop,
   * which only has the cumulative max_iter). No reference counterpart: it bounds frames
   * whose lagged-friction Newton iteration cycles instead of converging. */
  int max_iter_frame;
  /* 1: the first large cull of each narrow phase (pair cull, CCD) times its launch
   * variants on the same input and keeps the fastest for the handle (results do not
   * depend on the variant); 0: the default variants. No reference counterpart. */
  int autotune;
  /* 1: with solver 0, a scene whose Newton matrix is block-tridiagonal in body order
   * (contacts only between consecutive bodies: chains, stacks) is solved directly by a
   * block Cholesky of each run of linked bodies, as the reference's sparse direct solver
   * (Pardiso LLT, abd.cpp:233-264) would; other scenes take the PCG. 0: every scene takes
   * the PCG. No reference counterpart. */
  int tri_direct;
} abd_config;

/* Scene: bodies with their rest meshes (local vertex ids per body). */
typedef struct {
  int n_bodies;
  const double* q0;            /* n_bodies * 12 */
  const double* dqdt;          /* n_bodies * 12 */
  const double* mass;          /* n_bodies; < 0 marks a static body */
  const double* Ic;            /* n_bodies */
  const int* vert_off;         /* n_bodies + 1 */
  const double* rest_vertices; /* vert_off[n] * 3 */
  const int* edge_off;         /* n_bodies + 1 */
  const int* edges;            /* edge_off[n] * 2, local vertex ids */
  const int* face_off;         /* n_bodies + 1 */
  const int* faces;            /* face_off[n] * 3, local vertex ids */
  const int* scene_id;         /* n_bodies or NULL: bodies of different scenes never touch;
                                  bodies of one scene must be contiguous. Each scene runs
                                  its own Newton loop, CCD bound and line search, exactly as
                                  if it were stepped alone (the batched mode; the reference
                                  steps one scene per ABD object). */
} abd_scene_desc;

typedef struct {
  int frames, newton_iters, ls_trials, pcg_iters;
  int n_pt, n_ee, n_vg, n_overlaps; /* maxima over the frames */
  int status;
  int pad;
  long long kernel_launches;                        /* kernels launched by these frames */
  double toi_min, alpha_min;
  double t_ipc_ms, t_solver_ms, t_ccd_ms, t_ls_ms; /* reference's 4-phase breakdown */
  double bytes_moved;                               /* algorithmic bytes of the path */
  double device_ms;                                 /* CUDA-event time of the call on the handle's stream */
} abd_frame_stats;

typedef struct abd_handle abd_handle;

/* Replaces ABD(cubes, globals) (model/abd.h:13-14). */
int abd_create(const abd_scene_desc* scene, const abd_config* cfg, abd_handle** out);
/* Reads a reference config.json and scene JSON (test_cases/spinning_cube.cpp:56-127;
 * "obj" meshes resolved relative to the scene file). */
int abd_create_from_files(const char* config_json, const char* scene_json, abd_handle** out);
/* Replaces ABD::implicit_euler(dt) (model/abd.cpp:30): advances n_frames frames. */
int abd_step(abd_handle* h, double dt, int n_frames, abd_frame_stats* stats);
int abd_get_state(abd_handle* h, double* q0, double* qdot);
/* ---- traces and the viewer loop (view/control.cpp:41,84-90; view/model_view.cpp:282-295) ----
 * Frame files in the reference's binary layout (player_save / player_load,
 * model/mutils.cpp:257-276, 293-329): <folder>/<ts> holds, per body, q0 (p, a1, a2, a3)
 * then dqdt, as raw doubles. abd_create_from_files reads "trace_folder", "starting_ts"
 * (>= 0: the initial state is loaded from that frame file and the frame counter starts
 * there) and "ending_ts" of the config. */
int abd_trace_save(abd_handle* h, const char* folder, int ts, int init); /* init: recreate the folder,
                                                                            copy config and scene in */
int abd_trace_load(abd_handle* h, const char* folder, int ts);
/* Trace settings of the handle: folder, frame counter ts, starting_ts, ending_ts, and the
 * config / scene files a new trace folder receives (either may be NULL). */
int abd_set_trace(abd_handle* h, const char* folder, int ts, int starting_ts, int ending_ts, const char* config_json,
                  const char* scene_json);
int abd_get_trace(abd_handle* h, int* ts, int* starting_ts, int* ending_ts, char* folder, int folder_cap);
int abd_trace_files(abd_handle* h, const char** config_json, const char** scene_json);
/* The viewer loop without rendering: steps frame after frame until the frame counter
 * reaches ending_ts; with record != 0 each new state is saved as frame file <ts> (the
 * folder recreated on the pass that starts at ts 0, as the reference does). stats sums
 * the frames. */
int abd_run(abd_handle* h, int record, abd_frame_stats* stats);
int abd_set_state(abd_handle* h, const double* q0, const double* qdot);
int abd_get_counts(abd_handle* h, int* n_bodies, int* n_vertices, int* n_edges, int* n_faces);
/* Cumulative Newton counter (the reference's ABD::iter, model/abd.h:53); of scene 0 for
 * abd_get_iter, of every scene for abd_set_iter. */
int abd_get_iter(abd_handle* h);
int abd_set_iter(abd_handle* h, int iter);
/* Friction coefficient of the handle (config "mu"), e.g. between differentiated rollouts. */
int abd_set_friction(abd_handle* h, double mu);
int abd_get_friction(abd_handle* h, double* mu);
/* Adjoint of one converged frame (no reference counterpart: the reference has no
 * derivatives). The frame maps the frame-start state (q_t, v_t) and mu to q_{t+1}; given
 * gq_next = dL/dq_{t+1} it solves J^T w = gq_next with J the exact Jacobian of the frame's
 * optimality condition at q_{t+1} (no PSD projection, no damping; every friction
 * multiplier and tangent frame following the configuration, as the reference recomputes
 * them at each Newton iterate) by GMRES preconditioned with the forward Newton matrix,
 * and returns gq_t = dL/dq_t, gv_t = dL/dv_t and *gmu = dL/dmu (gmu may be NULL). All
 * arrays are n_bodies * 12 host doubles. */
int abd_adjoint_frame(abd_handle* h, const double* q_t, const double* v_t, const double* q_next,
                      const double* gq_next, double* gq_t, double* gv_t, double* gmu);
/* Autotuner choices of the handle: box-phase steps of the pair-cull and CCD narrow phases
 * (steps[0], steps[1]; 0 while not tuned) and the times of the three variants measured
 * when tuning (ms[0..2] pair cull, ms[3..5] CCD; 0 while not tuned). */
int abd_autotune_info(abd_handle* h, int* steps, double* ms);
/* GMRES iterations and final relative residual of the handle's last abd_adjoint_frame. */
int abd_adjoint_stats(abd_handle* h, int* iterations, double* rel_residual);
/* Batched mode (no reference counterpart: the reference steps one scene per ABD object).
 * Number of scenes of the handle, and per-scene counts (arrays of that length, any may be
 * NULL) accumulated over the frames of the last abd_step call, plus each scene's
 * cumulative Newton counter. */
int abd_get_scene_count(abd_handle* h);
int abd_get_scene_stats(abd_handle* h, int* newton_iters, int* ls_trials, int* pcg_iters, int* iter);
/* Message of the handle's last error; with h = NULL, of the last failing call without a
 * handle (abd_create*) made by the calling host thread. */
const char* abd_last_error(abd_handle* h);
void abd_destroy(abd_handle* h);
/* Per-kernel device timing: when enabled, every kernel of the step is bracketed with
 * CUDA events on the handle's stream. abd_kernel_times returns the number of kernel
 * classes (<= max_n), their names (32 chars each), total ms and launch counts since the
 * last abd_profile call. */
int abd_profile(abd_handle* h, int enable);
int abd_kernel_times(abd_handle* h, int max_n, char* names, double* total_ms, long long* launches);
/* As abd_kernel_times, plus each class's work units (pairs, candidates, rows, ...) and
 * algorithmic bytes (per-unit figure x units) over the same launches. */
int abd_kernel_work(abd_handle* h, int max_n, char* names, double* total_ms, long long* launches, double* units,
                    double* bytes);

/* ---- stage entry points (parity tests and profiling) ---- */
/* Culls at state q (+ dq): vtn 1 at q, 2 at q + dq, 3 the trajectory q -> q + dq.
 * counts[0..3] = pt, ee, vg pairs, overlaps; *toi is written for vtn 3. */
int abd_cull(abd_handle* h, int vtn, const double* q, const double* dq, int* counts, double* toi);
/* Pair set of the last vtn 1/2 cull: pt/ee tuples (body, prim, body, prim), types. */
int abd_get_pairs(abd_handle* h, int* pt, int* pt_type, int* ee, int* ee_type, int* vg);
/* Newton system at state q for the pair set culled at q: gradient (12 nb), diagonal
 * blocks (144 nb, row-major), upper off-diagonal blocks (keys I<J, 144 each). */
int abd_newton_system(abd_handle* h, const double* q, double* grad, double* diag, int* n_off, int* off_keys,
                      double* off_vals, int max_off);
/* Line-search energy (E_barrier_plus_inert energy.cpp:19-86, E_fric :195-258, E_ground
 * :261-270) at q + dq with the friction lagged at q, i.e. the first trial of
 * ABD::line_search at alpha = 1 (line_search.cpp:88-110), with the handle's q0 / qdot as
 * the frame start. Culls at q, assembles there (lagged tangent bases and multipliers),
 * culls at q + dq and evaluates. terms (6 per scene, or NULL): inertia + orthogonality,
 * point-triangle barrier, edge-edge barrier (mollified), ground barrier, friction, and the
 * scene total as the line search sums it. counts (6, or NULL): pt, ee, vg pairs of the set
 * at q + dq, then of the lagged set at q. Per-pair arrays (each NULL or sized by counts):
 * barrier energies of the set at q + dq, friction energies of the lagged set. */
int abd_energy(abd_handle* h, const double* q, const double* dq, double* terms, int* counts, double* e_pt,
               double* e_ee, double* e_vg, double* f_pt, double* f_ee, double* f_vg);
/* Newton step dq = -H^{-1} grad at state q (PCG). */
int abd_newton_dq(abd_handle* h, const double* q, double* dq, int* pcg_iters);

/* ---- per-primitive functions (the reference's python `abdtk` module,
 *      python/bindings.cpp:42-83), batched over n primitives ---- */
/* x: n * 12 (p, t0, t1, t2). type / dist optional (computed when type[i] < 0).
 * H: n * 144 row-major vertex-space Hessian, g: n * 12. */
int abd_ipc_hess_pt_batch(int n, const double* x, const int* type, const double* dist, double dhat, double kappa,
                          int psd, double* H, double* g);
int abd_ipc_hess_ee_batch(int n, const double* x, const int* type, const double* dist, double dhat, double kappa,
                          double eps_x, int psd, double* H, double* g, double* mollifier);
/* x: n * 24 (four points at t0 then four at t1). */
int abd_pt_collision_time_batch(int n, const double* x, double* toi);
int abd_ee_collision_time_batch(int n, const double* x, double* toi);
/* Distance type and squared distance; x: n * 12. */
int abd_pt_distance_batch(int n, const double* x, int* type, double* dist);
int abd_ee_distance_batch(int n, const double* x, int* type, double* dist);

/* Allocation-free minimum point-triangle time of impact. No counterpart in the
 * reference. For callers that cannot allocate device memory where they call it (inside
 * a CUDA-graph stream capture, or under a host framework whose pool allocator owns all
 * device memory): inputs and outputs are the caller's device buffers -- d_x (n * 24
 * doubles, as abd_pt_collision_time_batch), d_toi (n per-trajectory TOIs), d_min (the
 * minimum) -- and the only scratch is a fixed 256 kB array in this library's device
 * memory, shared by all calls (overlapping calls on the GPU race; serialise them).
 * n <= ABD_NOALLOC_MAX_N, else ABD_ERR_INVALID. The first call on each device looks the
 * scratch address up and must come before any stream capture. Work is queued on
 * `stream` (a cudaStream_t, NULL = default stream); the call does not synchronise. */
#define ABD_NOALLOC_MAX_N (1 << 22)
int abd_pt_min_toi_noalloc(int n, const double* d_x, double* d_toi, double* d_min, void* stream);
/* Message of the last failing abd_pt_min_toi_noalloc call made by the calling host thread. */
const char* abd_noalloc_last_error(void);

/* Dense FP64 FMA throughput of this GPU in GFLOP/s (roofline denominator for the
 * FP64-bound kernels; measured with a fixed independent-FMA kernel). */
double abd_measure_fp64_gflops(void);

#ifdef __cplusplus
}
#endif
#endif /* ABD_GB300_H */
