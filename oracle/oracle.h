/*
 * CPU oracle for the projective-dynamics (PD) cloth solve.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (the CUDA library under
 * cloth-cuda_gb300/) links, loads or calls this code.  Only tests/, the
 * smoke check in __graft_entry__.py and the CPU-baseline leg of bench.py use
 * it, and only to compare results with or as the timed CPU baseline.
 *
 * It restates, in plain C, the reference algorithms of Chongyao/cloth-cuda:
 *   generator          src/mesh_generator.cpp:6-91
 *   rest state         src/cloth_mesh.cpp:138-211
 *   topology           src/mesh_topology.cpp:11-97
 *   stretch/bend/diag  src/sim_constraints.cpp:16-192
 *   pins               src/constraints.cpp:14-41
 *   GPU step (literal) src/pd_solver.cu:18-434, 496-621
 *   CPU step (direct)  src/stretch_reference.cpp:27-280
 * plus the consistent Chebyshev-Jacobi PD step and the PD residual, which have
 * no reference counterpart (the reference never subtracts the off-diagonal
 * coupling in its Jacobi step and never applies its Chebyshev blend).
 *
 * Parity status: the setup stage is pinned by the reference's own invariants
 * (src/tests/test_mesh.cpp, test_topology.cpp, test_constraints.cpp) and the
 * literal step is pinned against the reference's own CUDA kernels compiled
 * from src/pd_solver.cu (golden fixtures under tests/golden/).  The reference
 * ships no golden vectors for the solve itself; the consistent step is pinned
 * only by known-answer tests and by agreement with the direct solve.
 */
#ifndef PDG_ORACLE_H
#define PDG_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Problem description shared by every solver routine.  Arrays are in the
 * caller's vertex order, AoS xyz. */
typedef struct orc_problem {
    int N, T, E;               /* vertices, triangles, bend hinges           */
    const int*   tris;         /* T*3                                        */
    const float* Dm_inv;       /* T*4 col-major 2x2: g00, g10, g01, g11      */
    const float* area;         /* T                                          */
    const float* k_stretch;    /* T                                          */
    const int*   hinge;        /* E*4  (v0, v1, v2, v3)                      */
    const float* hinge_w;      /* E*4  cotangent weights                     */
    const float* hinge_n;      /* E    rest curvature norm                   */
    const float* hinge_k;      /* E    bend stiffness                        */
    const float* mass;         /* N                                          */
    int          P;            /* pinned vertices                            */
    const int*   pin_idx;      /* P                                          */
    const float* pin_target;   /* P*3                                        */
    double h;                  /* time step                                  */
    double damping;            /* velocity damping, 0..1                     */
    double ext[3];             /* external acceleration (gravity + wind)     */
} orc_problem;

/* Settings of the consistent Chebyshev-Jacobi step. */
typedef struct orc_jacobi_opts {
    int    iters;      /* iteration cap                                     */
    double tol;        /* relative residual target; <= 0: run all iters     */
    int    use_cheb;   /* apply the Chebyshev blend                         */
    double rho;        /* spectral-radius estimate                          */
    int    delay;      /* Chebyshev delay S: omega = 1 while k < S          */
    double gamma;      /* under-relaxation of the Jacobi update             */
    int    init;       /* 0: inertial start y, 1: previous x, 2: given x0   */
} orc_jacobi_opts;

/* ---------------- setup (float, as the reference computes it) ---------- */
int  orc_grid_counts(int nrows, int ncols, int type, int* N, int* T);
void orc_generate_grid(int nrows, int ncols, float size, int type,
                       float* pos, int* tris);
void orc_rest_state(int N, int T, const float* pos, const int* tris,
                    float density, float* Dm_inv, float* area, float* mass,
                    float* dFdx /* T*54 row-major 6x9, may be NULL */);
/* Unique edges sorted by (v0, v1): rows of (v0, v1, tri_a, tri_b). */
int  orc_topology(int N, int T, const int* tris, int* edges /* 3T*4 */);
/* Bend hinges over inner edges in the order orc_topology returns them. */
int  orc_build_bend(int N, const float* pos, const int* tris, int nE,
                    const int* edges, float k, int* hinge, float* w,
                    float* n_rest, float* hk);
void orc_jacobi_diag(int N, int T, const int* tris, const float* Dm_inv,
                     const float* area, const float* k_stretch, int E,
                     const int* hinge, const float* w, const float* hk,
                     const float* mass, float h, float* diag);

/* ---------------- solve ------------------------------------------------- */
/* One frame with the semantics of the reference CUDA path. */
void orc_step_literal_f32(const orc_problem* p, const float* diag,
                          int iters, float* x, float* v);
/* One frame of consistent Chebyshev-Jacobi PD.  x, v in/out; x0 is read when
 * opts->init == 2.  res (iters+1 entries, may be NULL) receives the absolute
 * free-DOF residual norm of every iterate; *res_y the residual at y;
 * *used the number of Jacobi sweeps whose result was kept. */
void orc_step_jacobi_f64(const orc_problem* p, const double* diag,
                         const orc_jacobi_opts* o, double* x, double* v,
                         const double* x0, double* res, double* res_y,
                         int* used);
void orc_step_jacobi_f32(const orc_problem* p, const float* diag,
                         const orc_jacobi_opts* o, float* x, float* v,
                         const float* x0, double* res, double* res_y,
                         int* used);
/* Residual r(x) of the PD energy at x (free DOFs only); returns its norm. */
double orc_residual_f64(const orc_problem* p, const double* y,
                        const double* x, double* r /* N*3 or NULL */);
/* One frame of local/global PD with a sparse LDL^T global solve.
 * pin_elim 0: the reference's row/column zeroing, 1: consistent elimination.
 * with_bend 0 reproduces the reference CPU path (stretch only). */
int  orc_step_direct_f64(const orc_problem* p, int iters, int pin_elim,
                         int with_bend, double* x, double* v);
int  orc_step_direct_f32(const orc_problem* p, int iters, int pin_elim,
                         int with_bend, float* x, float* v);
/* Strictly lower entries of the last LDL^T factor the direct solve built
 * (3N x 3N, minimum-degree order). */
long long orc_last_factor_nnz(void);
/* Solve K z = b for the frame's global matrix (for the scipy cross-check). */
int  orc_global_matrix_f64(const orc_problem* p, int pin_elim, int with_bend,
                           int* nnz, int* ri, int* ci, double* val);

#ifdef __cplusplus
}
#endif
#endif
