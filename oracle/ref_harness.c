/*
 * Harness that runs the reference's own CUDA kernels -- TEST INFRASTRUCTURE ONLY.
 *
 * Loads oracle/_ref/pd_solver_ref.cubin (src/pd_solver.cu of the reference,
 * compiled by ref_build.py) with the CUDA driver API and launches its kernels
 * in the order of PDSolver::step (src/pd_solver.cu:496-621): copy x to prev,
 * predict, then per iteration stretch projection, bend projection, clear rhs,
 * stretch rhs, bend rhs, inertial rhs, Jacobi divide, pins; finally the
 * velocity update and pins.  Block size 256, legacy default stream, as the
 * reference.  Used only to produce golden vectors for the oracle and, in a
 * GPU test, to time the reference's kernels beside the fused sweep.
 */
#include <cuda.h>
#include <stdio.h>
#include <string.h>

#define NK 10
static const char* kNames[NK] = {
    "_Z14predict_kernel", "_Z26tri_stretch_project_kernel", "_Z33accumulate_tri_stretch_rhs_kernel",
    "_Z19bend_project_kernel", "_Z26accumulate_bend_rhs_kernel", "_Z16clear_rhs_kernel",
    "_Z23add_inertial_rhs_kernel", "_Z20jacobi_divide_kernel", "_Z22update_velocity_kernel",
    "_Z24apply_constraints_kernel"};
enum { K_PREDICT, K_TRI, K_TRI_RHS, K_BEND, K_BEND_RHS, K_CLEAR, K_INERT, K_DIV, K_VEL, K_PINS };

#define CHK(x)                                                                                  \
    do {                                                                                        \
        CUresult r_ = (x);                                                                      \
        if (r_ != CUDA_SUCCESS) {                                                               \
            const char* s_ = NULL;                                                              \
            cuGetErrorString(r_, &s_);                                                          \
            snprintf(err, (size_t)errlen, "%s failed: %s", #x, s_ ? s_ : "?");                  \
            rc = -1;                                                                            \
            goto done;                                                                          \
        }                                                                                       \
    } while (0)

static unsigned nb(int n) { return (unsigned)((n + 255) / 256); }

/* The reference's frame: its launches in PDSolver::step order.  ev0/ev1
 * (may be 0) are recorded around the iteration loop. */
typedef struct {
    CUfunction fn[NK];
    int N, T, E, P;
    CUdeviceptr pos, vel, mass, tris, G, area, k, diag, quads, bw, bn, bk, pins, tgt;
    CUdeviceptr pred, rhs, prev, nw, proj, bproj;
} RefFrame;

static CUresult ref_frame(RefFrame* f, int iters, float dt, float gravity, float damping, CUevent ev0, CUevent ev1)
{
    CUresult r;
    int N = f->N, T = f->T, E = f->E, P = f->P;
    const size_t b3 = sizeof(float) * 3 * (size_t)N;
    const float h2 = dt * dt;
#define L(x) do { r = (x); if (r != CUDA_SUCCESS) return r; } while (0)
    L(cuMemcpyDtoD(f->prev, f->pos, b3));
    { void* a[] = {&f->pos, &f->vel, &f->pred, &N, &dt, &gravity};
      L(cuLaunchKernel(f->fn[K_PREDICT], nb(N), 1, 1, 256, 1, 1, 0, 0, a, NULL)); }
    if (ev0) L(cuEventRecord(ev0, 0));
    CUdeviceptr d_in = f->pos, d_out = f->nw;
    for (int it = 0; it < iters; ++it) {
        if (T > 0) {
            void* a[] = {&d_in, &f->tris, &f->G, &f->proj, &T};
            L(cuLaunchKernel(f->fn[K_TRI], nb(T), 1, 1, 256, 1, 1, 0, 0, a, NULL));
        }
        if (E > 0) {
            void* a[] = {&d_in, &f->quads, &f->bw, &f->bn, &f->bproj, &E};
            L(cuLaunchKernel(f->fn[K_BEND], nb(E), 1, 1, 256, 1, 1, 0, 0, a, NULL));
        }
        { void* a[] = {&f->rhs, &N};
          L(cuLaunchKernel(f->fn[K_CLEAR], nb(N), 1, 1, 256, 1, 1, 0, 0, a, NULL)); }
        if (T > 0) {
            void* a[] = {&f->tris, &f->G, &f->area, &f->k, &f->proj, &f->rhs, &T, (void*)&h2};
            L(cuLaunchKernel(f->fn[K_TRI_RHS], nb(T), 1, 1, 256, 1, 1, 0, 0, a, NULL));
        }
        if (E > 0) {
            void* a[] = {&f->quads, &f->bw, &f->bk, &f->bproj, &f->rhs, &E, (void*)&h2};
            L(cuLaunchKernel(f->fn[K_BEND_RHS], nb(E), 1, 1, 256, 1, 1, 0, 0, a, NULL));
        }
        { void* a[] = {&f->rhs, &f->mass, &f->pred, &N};
          L(cuLaunchKernel(f->fn[K_INERT], nb(N), 1, 1, 256, 1, 1, 0, 0, a, NULL)); }
        { void* a[] = {&d_out, &f->rhs, &f->diag, &N};
          L(cuLaunchKernel(f->fn[K_DIV], nb(N), 1, 1, 256, 1, 1, 0, 0, a, NULL)); }
        if (P > 0) {
            void* a[] = {&d_out, &f->vel, &f->pins, &f->tgt, &P};
            L(cuLaunchKernel(f->fn[K_PINS], nb(P), 1, 1, 256, 1, 1, 0, 0, a, NULL));
        }
        { CUdeviceptr t = d_in; d_in = d_out; d_out = t; }
    }
    if (ev1) L(cuEventRecord(ev1, 0));
    if (d_in != f->pos) L(cuMemcpyDtoD(f->pos, d_in, b3));
    { void* a[] = {&f->prev, &f->vel, &f->pos, &N, &dt, &damping};
      L(cuLaunchKernel(f->fn[K_VEL], nb(N), 1, 1, 256, 1, 1, 0, 0, a, NULL)); }
    if (P > 0) {
        void* a[] = {&f->pos, &f->vel, &f->pins, &f->tgt, &P};
        L(cuLaunchKernel(f->fn[K_PINS], nb(P), 1, 1, 256, 1, 1, 0, 0, a, NULL));
    }
#undef L
    return CUDA_SUCCESS;
}

/* Loads the reference's kernels and uploads one cloth; `nframes` frames
 * follow.  With timing (frame_ms != NULL), `nframes` frames are timed after
 * one untimed frame, each from the input state (re-uploaded before it,
 * outside the timed region): frame_ms and loop_ms receive the mean time of a
 * whole frame and of its iteration loop (CUDA events on the legacy stream).
 * Without timing, the frames run one after another and the result is copied
 * back into pos / vel. */
static int ref_run(const char* cubin, int N, int T, int E, int P, float* pos, float* vel, const float* mass,
                   const int* tris, const float* Dm_inv, const float* rest_area, const float* stretch_k,
                   const float* diag, const int* quads, const float* bw, const float* bn, const float* bk,
                   const int* pins, const float* targets, int iters, float dt, float gravity, float damping,
                   int nframes, float* frame_ms, float* loop_ms, char* err, int errlen)
{
    int rc = 0;
    CUdevice dev;
    CUcontext ctx = NULL;
    CUmodule mod = NULL;
    CUevent e[4] = {0, 0, 0, 0};
    RefFrame f;
    memset(&f, 0, sizeof(f));
    f.N = N; f.T = T; f.E = E; f.P = P;
    const size_t b3 = sizeof(float) * 3 * (size_t)N;

    CHK(cuInit(0));
    CHK(cuDeviceGet(&dev, 0));
    CHK(cuDevicePrimaryCtxRetain(&ctx, dev));
    CHK(cuCtxSetCurrent(ctx));
    CHK(cuModuleLoad(&mod, cubin));
    {
        unsigned int count = 0;
        CHK(cuModuleGetFunctionCount(&count, mod));
        CUfunction all[64];
        if (count > 64) count = 64;
        CHK(cuModuleEnumerateFunctions(all, count, mod));
        for (unsigned int i = 0; i < count; ++i) {
            const char* name = NULL;
            CHK(cuFuncGetName(&name, all[i]));
            for (int k = 0; k < NK; ++k)
                if (name && strncmp(name, kNames[k], strlen(kNames[k])) == 0) f.fn[k] = all[i];
        }
        for (int k = 0; k < NK; ++k)
            if (!f.fn[k]) { snprintf(err, (size_t)errlen, "kernel %s not found", kNames[k]); rc = -2; goto done; }
    }
#define ALLOC_COPY(d, h, bytes) do { if ((bytes) > 0) { CHK(cuMemAlloc(&d, (bytes))); CHK(cuMemcpyHtoD(d, (h), (bytes))); } } while (0)
    ALLOC_COPY(f.pos, pos, b3);
    ALLOC_COPY(f.vel, vel, b3);
    ALLOC_COPY(f.mass, mass, sizeof(float) * (size_t)N);
    ALLOC_COPY(f.tris, tris, sizeof(int) * 3 * (size_t)T);
    ALLOC_COPY(f.G, Dm_inv, sizeof(float) * 4 * (size_t)T);
    ALLOC_COPY(f.area, rest_area, sizeof(float) * (size_t)T);
    ALLOC_COPY(f.k, stretch_k, sizeof(float) * (size_t)T);
    ALLOC_COPY(f.diag, diag, sizeof(float) * (size_t)N);
    ALLOC_COPY(f.quads, quads, sizeof(int) * 4 * (size_t)E);
    ALLOC_COPY(f.bw, bw, sizeof(float) * 4 * (size_t)E);
    ALLOC_COPY(f.bn, bn, sizeof(float) * (size_t)E);
    ALLOC_COPY(f.bk, bk, sizeof(float) * (size_t)E);
    ALLOC_COPY(f.pins, pins, sizeof(int) * (size_t)P);
    ALLOC_COPY(f.tgt, targets, sizeof(float) * 3 * (size_t)P);
    CHK(cuMemAlloc(&f.pred, b3));
    CHK(cuMemAlloc(&f.rhs, b3));
    CHK(cuMemAlloc(&f.prev, b3));
    CHK(cuMemAlloc(&f.nw, b3));
    if (T > 0) CHK(cuMemAlloc(&f.proj, sizeof(float) * 6 * (size_t)T));
    if (E > 0) CHK(cuMemAlloc(&f.bproj, sizeof(float) * 3 * (size_t)E));

    if (!frame_ms) {
        for (int q = 0; q < nframes; ++q) CHK(ref_frame(&f, iters, dt, gravity, damping, 0, 0));
        CHK(cuCtxSynchronize());
        CHK(cuMemcpyDtoH(pos, f.pos, b3));
        CHK(cuMemcpyDtoH(vel, f.vel, b3));
    } else {
        double tf = 0.0, tl = 0.0;
        for (int i = 0; i < 4; ++i) CHK(cuEventCreate(&e[i], CU_EVENT_DEFAULT));
        for (int q = -1; q < nframes; ++q) {
            CHK(cuMemcpyHtoD(f.pos, pos, b3));
            CHK(cuMemcpyHtoD(f.vel, vel, b3));
            CHK(cuEventRecord(e[0], 0));
            CHK(ref_frame(&f, iters, dt, gravity, damping, e[1], e[2]));
            CHK(cuEventRecord(e[3], 0));
            CHK(cuEventSynchronize(e[3]));
            float a = 0.f, b = 0.f;
            CHK(cuEventElapsedTime(&a, e[0], e[3]));
            CHK(cuEventElapsedTime(&b, e[1], e[2]));
            if (q >= 0) { tf += a; tl += b; }
        }
        *frame_ms = (float)(tf / (nframes > 0 ? nframes : 1));
        if (loop_ms) *loop_ms = (float)(tl / (nframes > 0 ? nframes : 1));
    }
done:
    for (int i = 0; i < 4; ++i)
        if (e[i]) cuEventDestroy(e[i]);
    {
        CUdeviceptr all[] = {f.pos, f.vel, f.mass, f.tris, f.G, f.area, f.k, f.diag, f.quads, f.bw, f.bn, f.bk,
                             f.pins, f.tgt, f.pred, f.rhs, f.prev, f.nw, f.proj, f.bproj};
        for (size_t i = 0; i < sizeof(all) / sizeof(all[0]); ++i)
            if (all[i]) cuMemFree(all[i]);
    }
    if (mod) cuModuleUnload(mod);
    if (ctx) cuDevicePrimaryCtxRelease(dev);
    return rc;
}

int ref_step(const char* cubin, int N, int T, int E, int P, float* pos, float* vel, const float* mass,
             const int* tris, const float* Dm_inv, const float* rest_area, const float* stretch_k,
             const float* diag, const int* quads, const float* bw, const float* bn, const float* bk,
             const int* pins, const float* targets, int iters, float dt, float gravity, float damping,
             char* err, int errlen)
{
    return ref_run(cubin, N, T, E, P, pos, vel, mass, tris, Dm_inv, rest_area, stretch_k, diag, quads, bw, bn, bk,
                   pins, targets, iters, dt, gravity, damping, 1, NULL, NULL, err, errlen);
}

/* Timing of the reference's frame: the mean of `nframes` frames from the
 * input state (not changed), after one untimed frame. */
int ref_time(const char* cubin, int N, int T, int E, int P, float* pos, float* vel, const float* mass,
             const int* tris, const float* Dm_inv, const float* rest_area, const float* stretch_k,
             const float* diag, const int* quads, const float* bw, const float* bn, const float* bk,
             const int* pins, const float* targets, int iters, float dt, float gravity, float damping,
             int nframes, float* frame_ms, float* loop_ms, char* err, int errlen)
{
    if (!frame_ms || nframes <= 0) { snprintf(err, (size_t)errlen, "ref_time: bad arguments"); return -3; }
    return ref_run(cubin, N, T, E, P, pos, vel, mass, tris, Dm_inv, rest_area, stretch_k, diag, quads, bw, bn, bk,
                   pins, targets, iters, dt, gravity, damping, nframes, frame_ms, loop_ms, err, errlen);
}
