/*
 * pdg.h -- C ABI of the GB300-native projective-dynamics (PD) cloth solver.
 *
 * Drop-in boundary for the per-frame solve of Chongyao/cloth-cuda.  Every
 * entry point takes plain pointers and sizes, returns an int status
 * (PDG_OK = 0, negative on error; pdg_last_error_string() explains the last
 * failure on the calling thread) and never exits the process.  The reference
 * interface each group replaces is cited beside it.
 *
 * Vertex arrays crossing this boundary are AoS xyz float32 in the caller's
 * vertex order.  Internally the solver keeps a reordered float4 layout (compact
 * patches by recursive coordinate bisection, Z-order inside a patch);
 * the permutation never leaves the library.
 *
 * Threading: one host thread per handle.  Work is stream-ordered on the
 * stream given at creation (NULL = the legacy default stream, as in the
 * reference); host-pointer getters synchronise that stream.
 */
#ifndef PDG_H
#define PDG_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PDG_OK              0
#define PDG_ERR_ARG        -1   /* invalid argument or size                 */
#define PDG_ERR_CUDA       -2   /* a CUDA call failed                       */
#define PDG_ERR_ALLOC      -3   /* host or device allocation failed          */
#define PDG_ERR_STATE      -4   /* call out of order (e.g. no constraints)  */
#define PDG_ERR_TIMEOUT    -5   /* a bounded device wait gave up             */
#define PDG_ERR_NUMERIC    -6   /* NaN/Inf detected in the solve             */
#define PDG_ERR_IO         -7   /* file could not be read                    */

/* Global step of the solve. */
#define PDG_MODE_CONSISTENT        0  /* x += gamma D^-1 (b - K x), Chebyshev blend */
#define PDG_MODE_REFERENCE_LITERAL 1  /* x = rhs / diag as src/pd_solver.cu:385-398 */

/* Initial iterate of a frame. */
#define PDG_INIT_INERTIAL 0   /* y = x + h v + h^2 a, pins at their targets */
#define PDG_INIT_PREVIOUS 1   /* x_n (what src/pd_solver.cu:528 does)      */
#define PDG_INIT_WARMSTART 2  /* the learned prediction, kept only if its
                                 residual is below the inertial start's     */
#define PDG_INIT_WARMSTART_KEEP 3  /* the learned prediction, always kept (no
                                 residual judge; for evaluating the network:
                                 a trajectory that always keeps a prediction
                                 close to the previous frame's offset gains
                                 energy when its frames stop at a tolerance) */

/* Launch structure of the iteration loop. */
#define PDG_KERNEL_AUTO       0  /* resident when it fits, else the streaming
                                    kernel (no timing)                       */
#define PDG_KERNEL_GRAPH      1  /* one fused launch per iteration, frame in a CUDA graph */
#define PDG_KERNEL_PERSISTENT 2  /* one cooperative launch per frame, bounded grid barrier */
#define PDG_KERNEL_RESIDENT   3  /* persistent, one patch per block, records kept on chip */
#define PDG_KERNEL_AUTOTUNE   4  /* time every launch plan that fits (launch
                                    structure, patch size, threads per block)
                                    on this problem and keep the fastest;
                                    the choice is cached per device and
                                    problem shape for the process           */
#define PDG_KERNEL_STREAM     5  /* one launch per iteration (CUDA graph) on a
                                    persistent grid; each block stages its
                                    next patch's vertex data with bulk (TMA)
                                    and asynchronous copies while it solves
                                    the current one                          */

/* Solver configuration.  Mirrors PDSolverConfig (include/pd_solver.h:4-15);
 * fields after `damping` extend it. */
typedef struct pdg_config {
    int   max_iterations;     /* iteration cap per frame (50)                 */
    float tolerance;          /* relative residual target; <= 0: run the cap  */
    int   use_chebyshev;      /* Chebyshev blend (1)                          */
    float rho;                /* spectral-radius estimate (0.9)               */
    float gravity;            /* acceleration along y (-9.8)                  */
    float dt;                 /* time step (0.01)                             */
    float stretch_stiffness;  /* informational, as in the reference (1.0)     */
    float bend_stiffness;     /* informational, as in the reference (0.0)     */
    float damping;            /* velocity damping 0..1 (0)                    */
    /* ---- extensions ---- */
    float wind[3];            /* constant extra acceleration (0,0,0)          */
    int   cheb_delay;         /* omega = 1 while k < cheb_delay (1)           */
    float gamma;              /* under-relaxation of the Jacobi update (1)    */
    int   mode;               /* PDG_MODE_* (CONSISTENT)                      */
    int   init;               /* PDG_INIT_* (INERTIAL)                        */
    int   kernel;             /* PDG_KERNEL_* (AUTO)                          */
    int   patch_verts;        /* owned vertices per patch, 0 = solver's choice */
    int   block_threads;      /* threads per patch block, 0 = solver's choice  */
    int   compute_final_residual; /* evaluate r(x) of the returned iterate (1) */
    int   smem_carveout;      /* per-sweep kernels: percent of the unified
                                 L1/shared capacity given to shared memory
                                 (1-100); 0 = the CUDA runtime's choice (0) */
} pdg_config;

/* Per-frame statistics (one per cloth). */
typedef struct pdg_frame_stats {
    int    iterations;        /* Jacobi sweeps whose result was kept          */
    int    converged;         /* final relative residual <= tolerance         */
    int    warm_start_used;   /* learned start kept (1) or discarded (0)      */
    int    status;            /* PDG_OK or an error code for this cloth       */
    double res_inertial;      /* ||r(y_pinned)|| over free DOFs               */
    double res_initial;       /* ||r(x^0)||                                    */
    double res_final;         /* ||r(x returned)|| (if computed, else -1)     */
    double rel_residual;      /* res_final / res_inertial                      */
} pdg_frame_stats;

typedef struct pdg_mesh        pdg_mesh;         /* ClothMesh (include/cloth_mesh.h:18-67)          */
typedef struct pdg_constraints pdg_constraints;  /* SimConstraints + Constraints                    */
typedef struct pdg_solver      pdg_solver;       /* PDSolver (include/pd_solver.h:30-71), 1..n cloths */
typedef struct pdg_warmstart   pdg_warmstart;    /* learned warm start (no reference counterpart)   */

const char* pdg_last_error_string(void);
const char* pdg_version(void);
int  pdg_config_default(pdg_config* cfg);

/* ---------------- mesh: include/cloth_mesh.h:18-67 ----------------------- */
/* ClothMesh::precompute_rest_state (src/cloth_mesh.cpp:138-211) on a caller
 * mesh: rest_xyz N*3, tris T*3 (0-based). */
int  pdg_mesh_create(const float* rest_xyz, int N, const int* tris, int T,
                     float density, pdg_mesh** out);
/* generate_square_cloth (src/mesh_generator.cpp:6-91): x-z plane, `size` =
 * cell edge, type 0..3; then precompute_rest_state(density). */
int  pdg_mesh_generate(int nrows, int ncols, float size, int type,
                       float density, pdg_mesh** out);
/* Square cloth hanging in the x-y plane: row 0 on top at y = 0, rows going
 * down, cell = side/(n-1), z jitter N(0, jitter) from `seed`. */
int  pdg_mesh_generate_hanging(int nrows, int ncols, float side, int type,
                               float jitter, unsigned long long seed,
                               float density, pdg_mesh** out);
/* ClothMesh::load_obj (src/cloth_mesh.cpp:89-132): v / f records, 1-based,
 * polygons fan-triangulated. */
int  pdg_mesh_load_obj(const char* path, float density, pdg_mesh** out);
int  pdg_mesh_counts(const pdg_mesh* m, int* N, int* T);
/* Copy out rest positions, triangles, Dm_inv (T*4 col-major), rest area,
 * lumped mass and dF/dx (T*54, row-major 6x9).  Any pointer may be NULL. */
int  pdg_mesh_get(const pdg_mesh* m, float* rest_xyz, int* tris, float* Dm_inv,
                  float* area, float* mass, float* dFdx);
void pdg_mesh_destroy(pdg_mesh* m);

/* ---------------- topology: MeshTopology::build (src/mesh_topology.cpp:11-97) */
int  pdg_topology_counts(const pdg_mesh* m, int* num_edges, int* num_inner);
/* edges: rows (v0, v1, tri_a, tri_b) sorted by (v0, v1), v0 < v1, tri_b = -1
 * on the boundary; rest_len per edge; vert_tri_ptr N+1 / vert_tri (3T)
 * vertex->triangle adjacency; tri_tri T*3 neighbour opposite each corner
 * (-1 if none).  Any pointer may be NULL. */
int  pdg_topology_get(const pdg_mesh* m, int* edges, float* rest_len,
                      int* vert_tri_ptr, int* vert_tri, int* tri_tri);

/* ---------------- constraints: SimConstraints (include/sim_constraints.h:30-78)
 *                  and Constraints (include/constraints.h:5-36) ----------- */
int  pdg_constraints_create(const pdg_mesh* m, pdg_constraints** out);
/* SimConstraints::build_stretch (src/sim_constraints.cpp:16-22) */
int  pdg_constraints_build_stretch(pdg_constraints* c, float stiffness);
int  pdg_constraints_set_stretch_k(pdg_constraints* c, const float* k_per_tri);
/* SimConstraints::build_bend (src/sim_constraints.cpp:48-127) */
int  pdg_constraints_build_bend(pdg_constraints* c, float stiffness);
/* Constraints::set_from_list / pin_top_row / pin_corners
 * (src/constraints.cpp:14-41); targets NULL = rest positions. */
int  pdg_constraints_set_pins(pdg_constraints* c, const int* idx, int P,
                              const float* targets);
int  pdg_constraints_pin_top_row(pdg_constraints* c, int ncols);
int  pdg_constraints_pin_corners(pdg_constraints* c, int ncols);
int  pdg_constraints_counts(const pdg_constraints* c, int* num_bend, int* num_pins);
/* Bend hinges (v0,v1,v2,v3), weights w0..w3, rest norm, stiffness; pins and
 * targets.  Any pointer may be NULL. */
int  pdg_constraints_get(const pdg_constraints* c, float* stretch_k, int* quads,
                         float* w, float* n_rest, float* bend_k, int* pins,
                         float* targets);
/* SimConstraints::precompute_jacobi_diag (src/sim_constraints.cpp:133-192) */
int  pdg_constraints_jacobi_diag(const pdg_constraints* c, float dt, float* diag);
void pdg_constraints_destroy(pdg_constraints* c);

/* ---------------- solver: PDSolver (include/pd_solver.h:30-71) ------------ */
/* PDSolver::PDSolver (src/pd_solver.cu:445-460).  The mesh and constraints
 * are copied; they may be destroyed afterwards.  stream = cudaStream_t or
 * NULL.  Initial state: x = rest positions, v = 0 (ClothMesh::upload_to_gpu,
 * src/cloth_mesh.cpp:31-83). */
int  pdg_solver_create(const pdg_config* cfg, const pdg_mesh* m,
                       const pdg_constraints* c, void* stream, pdg_solver** out);
/* Many cloths of uneven size in one solver (one persistent launch / graph per
 * frame).  cfgs: one per cloth (dt, gravity, wind, damping, rho, tolerance,
 * cap may differ; the launch fields of cfgs[0] apply to all). */
int  pdg_solver_create_batch(int ncloths, const pdg_config* cfgs,
                             const pdg_mesh* const* meshes,
                             const pdg_constraints* const* cons, void* stream,
                             pdg_solver** out);
/* Host-side check of the patch layout a solver builds for these cloths with
 * `patch_verts`-vertex patches; needs no GPU.  It checks the vertex reorder
 * and partition, the halo and neighbour lists, that every owned vertex
 * another patch reads comes first (boundary vertices), that every
 * contribution slot of an owned vertex is written exactly once (for a
 * boundary vertex, by the records before its sum), and that every triangle
 * through an owned vertex is held by the patch.  PDG_OK with a summary in
 * *info; PDG_ERR_STATE with the first violation in pdg_last_error_string();
 * PDG_ERR_ARG for bad arguments.  No counterpart in the reference. */
typedef struct pdg_layout_info {
    int       vertices, patches, max_owned, max_local;
    long long halo_total;      /* halo entries over all patches            */
    long long boundary_total;  /* owned vertices that other patches read   */
    long long cells;           /* cell records (triangle pairs)            */
    long long phase_a_cells;   /* cell records through boundary vertices   */
    long long lone_hinges;     /* bend hinges that no cell holds           */
    long long smem_resident;   /* resident kernel: shared bytes per patch  */
} pdg_layout_info;
int  pdg_layout_check(int ncloths, const pdg_config* cfgs,
                      const pdg_mesh* const* meshes,
                      const pdg_constraints* const* cons, int patch_verts,
                      pdg_layout_info* info);
/* The same check after planting one mistake in the built layout, so that a
 * test can show the checker catches it: 1 two vertices' caller indices
 * swapped, 2 a halo entry repeated, 3 a boundary vertex moved past the
 * published prefix, 4 two records pointed at one contribution slot, 5 a
 * cell dropped, 6 a halo entry out of range.  PDG_ERR_STATE with the
 * violation when caught; PDG_ERR_ARG if the layout has no place for it. */
int  pdg_layout_check_planted(int ncloths, const pdg_config* cfgs,
                              const pdg_mesh* const* meshes,
                              const pdg_constraints* const* cons, int patch_verts,
                              int mistake, pdg_layout_info* info);
int  pdg_solver_num_cloths(const pdg_solver* s, int* n);
int  pdg_solver_cloth_counts(const pdg_solver* s, int cloth, int* N, int* T);
/* PDSolver::step (src/pd_solver.cu:496-621): `nframes` frames.  stats: NULL
 * or ncloths entries describing the last frame (reading them synchronises). */
int  pdg_solver_step(pdg_solver* s, int nframes, pdg_frame_stats* stats);
/* PDSolver::reset (src/pd_solver.cu:491-494): restart the Chebyshev state. */
int  pdg_solver_reset(pdg_solver* s);
/* State of one cloth, AoS xyz float32 in its own vertex order.  x or v may be
 * NULL.  on_device != 0: pointers are device pointers (stream-ordered copy),
 * else host pointers (the copy synchronises). */
int  pdg_solver_set_state(pdg_solver* s, int cloth, const float* x,
                          const float* v, int on_device);
int  pdg_solver_get_state(pdg_solver* s, int cloth, float* x, float* v,
                          int on_device);
/* Whole batch at once: x, v hold sum(N) vertices, cloths back to back. */
int  pdg_solver_set_state_all(pdg_solver* s, const float* x, const float* v, int on_device);
int  pdg_solver_get_state_all(pdg_solver* s, float* x, float* v, int on_device);
/* A frame loop's upload / step / download in one call, host buffers, whole
 * batch in caller order (as the _all calls).  x_in / v_in (either may be
 * NULL: keep the solver's state) are copied in, nframes frames run, the
 * result is copied into x_out / v_out (either may be NULL), and the call
 * returns once the copies are complete, after one synchronisation.  The
 * same as set_state_all + step + get_state_all, without their separate
 * synchronisations.  Replaces the step + cudaMemcpy of mesh.d_pos / d_vel
 * in the reference's frame loop (src/tools/sim_cloth.cpp:237-251 with
 * lines 44-45 and 82-83).  stats as for pdg_solver_step.  With the
 * resident kernel the frame launch itself reads the inputs and writes the
 * outputs (page-locked buffers in place); a wait that runs out leaves the
 * outputs undefined, like the solver state. */
int  pdg_solver_step_host(pdg_solver* s, int nframes, const float* x_in, const float* v_in,
                          float* x_out, float* v_out, pdg_frame_stats* stats);
/* Relative-residual target of one cloth (cloth = -1: every cloth), as
 * pdg_config.tolerance at creation; 0 runs the sweep cap. */
int  pdg_solver_set_tolerance(pdg_solver* s, int cloth, float tolerance);
/* Replace the pin set of one cloth on a live solver (Constraints::set_from_list
 * + upload_to_gpu, src/constraints.cpp:14-22 and 77-101): idx P distinct
 * vertex indices of the cloth, targets P*3 (NULL = rest positions).  The
 * patch layout does not depend on the pins; only the per-vertex records
 * change.  An attached network reads the new pins from the next frame on;
 * its energy-norm loss weights (training only) keep the old ones until it is
 * attached again. */
int  pdg_solver_set_pins(pdg_solver* s, int cloth, const int* idx, int P, const float* targets);
/* Move the pins of one cloth (Constraints::target_positions). */
int  pdg_solver_set_pin_targets(pdg_solver* s, int cloth, const float* targets);
/* Inertial prediction y of the last frame and the residual r(x) of a given
 * state against it (host arrays, caller order), for diagnostics/tests. */
int  pdg_solver_get_prediction(pdg_solver* s, int cloth, float* y);
/* Kernel launches issued so far (fused iteration, predict, finalize, ...). */
int  pdg_solver_launch_count(const pdg_solver* s, long long* n);
/* Measurement helper: runs `nframes` frames as individual launches (no
 * graph) and times them with CUDA events on the solver's stream.  frame_ms:
 * average frame; sweep_ms: average duration of one fused sweep (the events
 * bracket the sweep launches; persistent kernel: frame time / sweeps). */
int  pdg_solver_time_frames(pdg_solver* s, int nframes, float* frame_ms, float* sweep_ms);
/* Wait budget (GPU clock cycles) of every grid-barrier / neighbour / copy
 * wait in the persistent, resident and streaming kernels (default 2e9,
 * about 1 s).  When a wait
 * runs out the kernel records an error and every block leaves at its next
 * wait.  The error stays recorded (later frames of the same call leave at
 * their first barrier) until pdg_solver_step with stats or
 * pdg_solver_time_frames reports it as PDG_ERR_TIMEOUT and clears it; the
 * solver state is then undefined until pdg_solver_set_state. */
int  pdg_solver_set_wait_budget(pdg_solver* s, long long cycles);
/* Test hook for the resident kernel's neighbour exchange: the tag number the
 * next frame starts from.  Each frame's exchanged offsets carry 32-bit tags
 * from a device word that every frame advances by its sweep count; a frame
 * whose tags would pass 2^32 - 1 first clears its patches' exchange words
 * and starts again from 0.  Setting a base near 2^32 makes the next frames
 * take that path.  No effect on the other kernels. */
int  pdg_solver_set_frame_tag(pdg_solver* s, unsigned long long tag);
/* Stream the solver works on (a cudaStream_t). */
int  pdg_solver_stream(const pdg_solver* s, void** stream);
/* Launch shape the solver picked: kernel (PDG_KERNEL_*), patch_verts,
 * block_threads, number of patches. */
int  pdg_solver_launch_info(const pdg_solver* s, int* kernel, int* patch_verts,
                            int* block_threads, int* npatches);
void pdg_solver_destroy(pdg_solver* s);

/* ---------------- autotuner (no counterpart in the reference) -------------
 * PDG_KERNEL_AUTOTUNE creates the solver once per candidate launch plan,
 * runs one untimed and three timed frames from the rest state (CUDA events
 * on the solver's stream), and builds the final solver with the fastest
 * plan.  Every plan computes bitwise the same iterates, so the choice
 * changes the speed only.  The candidate table is kept in the solver. */
typedef struct pdg_tune_entry {
    int   kernel;             /* PDG_KERNEL_GRAPH/_PERSISTENT/_RESIDENT/_STREAM */
    int   patch_verts;        /* owned vertices per patch                     */
    int   block_threads;      /* threads per block                            */
    float frame_ms;           /* mean frame time; < 0: plan does not fit      */
    int   chosen;             /* 1 for the plan the solver runs               */
    int   cached;             /* 1 when the choice came from the cache        */
} pdg_tune_entry;
/* Copies up to `cap` entries of the candidate table; *n = table size (0 for
 * solvers not created with PDG_KERNEL_AUTOTUNE). */
int  pdg_solver_tune_results(const pdg_solver* s, pdg_tune_entry* out, int cap, int* n);
/* Forgets every cached choice of this process. */
void pdg_autotune_clear_cache(void);

/* ---------------- learned warm start (no counterpart in the reference) ----
 * A 2-layer mesh message-passing network (hidden 64, bf16 weights and
 * activations, fp32 accumulation) predicts each vertex's offset x* - y of
 * the converged position from the inertial prediction.  Node features (14):
 * (y - x_n)/s, h v_n/s, pinned flag, log mass, log stretch k, log bend k, the
 * previous frame's offset d_prev/s and its validity flag (s = 2.725e-3 m,
 * one frame's gravity drop at h = 1/60).  The network's output is the change
 * of the offset: the prediction is d_prev + s out (a skip connection kept in
 * fp32).  d_prev is the offset x_n - y_(n-1) the solver kept at the end of
 * its previous frame; it is valid for a vertex whose state entering the frame
 * is bitwise the state the solver left (pdg_solver_set_state* and
 * pdg_solver_step_host inputs that change a vertex invalidate it, as does
 * attaching a network).  Edge features (4): log rest length and the current
 * edge vector over the rest length.
 *
 * Attached to a solver whose cloths use cfg.init = PDG_INIT_WARMSTART,
 * every frame judges the prediction against the inertial start and keeps,
 * per cloth, the better one (plain PD remains both fallback and judge):
 * with K = pdg_warmstart_set_judge_sweeps (default 1) > 0 both starts run K
 * sweeps on their own iterates and the cloth continues from the one whose
 * last evaluated residual, that of its iterate after K - 1 sweeps, is lower
 * (ties: the inertial start).  K = 1 compares the two starts' own residuals,
 * evaluated by each chain's first sweep; K = 0 compares them by a separate
 * evaluation before any sweep.  PDG_INIT_WARMSTART_KEEP always keeps
 * the prediction.  Parameter layout: see pdg_warmstart_get_params
 * (We[64][14] be[64] {A[64][64] B[64][64] C[64][4] c[64] U[64][128] u[64]}
 * x 2 Wd[3][64] bd[3], fp32). */
/* A new network from `seed`: random hidden layers and a zero decoder, so
 * that before training it predicts the previous frame's offset. */
int  pdg_warmstart_create(unsigned long long seed, pdg_warmstart** out);
int  pdg_warmstart_param_count(const pdg_warmstart* w, int* n);
int  pdg_warmstart_get_params(pdg_warmstart* w, float* host);
int  pdg_warmstart_set_params(pdg_warmstart* w, const float* host);
/* Forward + backward on a caller graph (host arrays): x N*14 node features,
 * symmetric CSR ptr (N+1) / adj, ef 4 features per directed edge, target
 * N*3, free weights N, ew one weight per directed edge of the loss's edge
 * term (NULL: 1).  Returns out N*3, the loss and the gradients (param_count
 * floats).  Not while attached to a solver. */
int  pdg_warmstart_eval(pdg_warmstart* w, int N, const float* x, const int* ptr, const int* adj,
                        const float* ef, const float* target, const float* freew, const float* ew,
                        float* out, float* loss, float* grads);
/* One Adam step (beta 0.9/0.999) with the gradients of the last eval/train. */
int  pdg_warmstart_adam_step(pdg_warmstart* w, float lr);
/* Bind to a solver (per-sweep kernels); its frames then use the prediction
 * for cloths with cfg.init == PDG_INIT_WARMSTART or _KEEP. */
int  pdg_warmstart_attach(pdg_warmstart* w, pdg_solver* s);
/* Training on data the solver generates: one frame of `s` from its current
 * state, then one Adam step (lr > 0) on (x_n, v_n, y, d_prev) ->
 * (x_{n+1} - y - d_prev). */
int  pdg_warmstart_train_frame(pdg_warmstart* w, pdg_solver* s, float lr, float* loss);
/* Training on a trajectory of `traj` (the network attached to it) with the
 * targets of a deeper solve: `deep` solves the same cloths with the same
 * vertex layout (created from the same meshes, constraints and launch plan,
 * with a larger cap or a lower tolerance).  One step copies traj's state
 * into `deep`, runs one frame of `deep` (the target x*), one frame of `traj`
 * (the trajectory and its kept offsets advance as in use), then one Adam
 * step (lr > 0) on (x_n, v_n, y, d_prev of traj) -> (x* - y - d_prev). */
int  pdg_warmstart_train_pair(pdg_warmstart* w, pdg_solver* traj, pdg_solver* deep, float lr, float* loss);
/* Loss of training and evaluation: mean squared offset error plus lambda/2
 * times the weighted squared error differences over the mesh's edges
 * (default 0).  The second term weighs the high-frequency part of the
 * error, which the residual of a start amplifies. */
int  pdg_warmstart_set_smoothness(pdg_warmstart* w, float lambda);
/* Edge weights of that term when training on an attached solver: 0 (default)
 * 1 per edge; 1 the energy norm e^T (M + K) e / m of the error, K the PD
 * system's stiffness approximated by a graph Laplacian with K's diagonal
 * (the Jacobi diagonal minus the mass). */
int  pdg_warmstart_set_energy_norm(pdg_warmstart* w, int enable);
/* Sweeps K each start runs before the judge (0..1000; default 1; at most
 * the sweep cap is used).  On held-out cloths of the batched distribution
 * K = 1, 2, 4 and 6 saved the same sweeps (within 1 %), so the default is
 * the cheapest. */
int  pdg_warmstart_set_judge_sweeps(pdg_warmstart* w, int sweeps);
int  pdg_warmstart_get_judge_sweeps(const pdg_warmstart* w, int* sweeps);
/* Measurement helper: mean device time (CUDA events on the attached
 * solver's stream) of the prediction for the solver's current state --
 * features, network forward and start offsets -- over `reps` runs after one
 * untimed run.  The solver's state is not changed. */
int  pdg_warmstart_time_inference(pdg_warmstart* w, int reps, float* ms);
void pdg_warmstart_destroy(pdg_warmstart* w);

/* ---------------- allocation-free frame ----------------------------------
 * No counterpart in the reference.  One frame of the consistent solve (the
 * arithmetic of pdg_solver_step, results equal to rounding) for callers that
 * cannot call cudaMalloc: applications that own all device memory through
 * their own pool and load this library as a plugin, and real-time loops that
 * cannot afford the device-wide synchronisation of cudaMalloc/cudaFree.
 * Inputs are the cloth in the reference's own device layout -- the arrays of
 * ClothMesh (pos, vel, mass, tris, Dm_inv, rest area), SimConstraints
 * (stretch k, Jacobi diagonal for cfg->dt, bend quads/w/n/k) and Constraints
 * (pin indices and targets); d_pos and d_vel are updated in place.  Every
 * vertex index (tris, quads, pins) must be < N, as in the reference's
 * arrays; indices are not checked on the device.  It allocates nothing: its
 * work arrays live in one static device array of about 8.4 MB that every GPU
 * loading the library keeps until exit, so N is limited to
 * PDG_NOALLOC_MAX_VERTS and the sweep count to PDG_NOALLOC_MAX_ITERS (larger
 * sizes return PDG_ERR_ARG).  The first call on a device looks up the
 * array's device address; make it before any stream capture.  The calling
 * thread's current device must own `stream` (checked) and the arrays.  All
 * calls share the array: calls that overlap on the GPU (other streams or host
 * threads) race.  Only PDG_MODE_CONSISTENT with PDG_INIT_INERTIAL.  stats:
 * NULL or one host struct (filling it synchronises the stream).  A frame
 * whose solve produced NaN/Inf keeps x, zeroes v and re-applies the pins;
 * it is reported only through stats->status (PDG_ERR_NUMERIC): the call
 * itself returns PDG_OK, since without stats it does not wait for the GPU. */
#define PDG_NOALLOC_MAX_VERTS 131072
#define PDG_NOALLOC_MAX_ITERS 4096
int  pdg_step_noalloc(const pdg_config* cfg, int N, float* d_pos, float* d_vel, const float* d_mass,
                      const float* d_jacobi_diag, int T, const int* d_tris, const float* d_Dm_inv,
                      const float* d_rest_area, const float* d_stretch_k, int E, const int* d_bend_quads,
                      const float* d_bend_w, const float* d_bend_n, const float* d_bend_k, int P,
                      const int* d_pin_idx, const float* d_pin_target, void* stream,
                      pdg_frame_stats* stats);

/* launch_apply_constraints_kernel (include/pd_solver.h:74-77): set
 * d_pos[idx] = target and d_vel[idx] = 0 for P pinned vertices, AoS xyz
 * device arrays, on `stream`. */
int  pdg_apply_pins(float* d_pos, float* d_vel, const int* d_indices,
                    const float* d_target, int num_pinned, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* PDG_H */
