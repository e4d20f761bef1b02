/*
 * Harness that runs the reference's own CUDA kernels -- TEST INFRASTRUCTURE ONLY.
 *
 * Loads oracle/_ref/pd_solver_ref.cubin (src/pd_solver.cu of the reference,
 * compiled by ref_build.py) with the CUDA driver API and launches its kernels
 * in the order of PDSolver::step (src/pd_solver.cu:496-621): copy x to prev,
 * predict, then per iteration stretch projection, bend projection, clear rhs,
 * stretch rhs, bend rhs, inertial rhs, Jacobi divide, pins; finally the
 * velocity update and pins.  Block size 256, legacy default stream, as the
 * reference.  Used only to produce golden vectors for the oracle.
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

int ref_step(const char* cubin, int N, int T, int E, int P, float* pos, float* vel, const float* mass,
             const int* tris, const float* Dm_inv, const float* rest_area, const float* stretch_k,
             const float* diag, const int* quads, const float* bw, const float* bn, const float* bk,
             const int* pins, const float* targets, int iters, float dt, float gravity, float damping,
             char* err, int errlen)
{
    int rc = 0;
    CUdevice dev;
    CUcontext ctx = NULL;
    CUmodule mod = NULL;
    CUfunction fn[NK];
    CUdeviceptr d_pos = 0, d_vel = 0, d_mass = 0, d_tris = 0, d_G = 0, d_area = 0, d_k = 0, d_diag = 0;
    CUdeviceptr d_quads = 0, d_bw = 0, d_bn = 0, d_bk = 0, d_pins = 0, d_tgt = 0;
    CUdeviceptr d_pred = 0, d_rhs = 0, d_prev = 0, d_new = 0, d_proj = 0, d_bproj = 0;
    const size_t b3 = sizeof(float) * 3 * (size_t)N;
    memset(fn, 0, sizeof(fn));

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
                if (name && strncmp(name, kNames[k], strlen(kNames[k])) == 0) fn[k] = all[i];
        }
        for (int k = 0; k < NK; ++k)
            if (!fn[k]) { snprintf(err, (size_t)errlen, "kernel %s not found", kNames[k]); rc = -2; goto done; }
    }
#define ALLOC_COPY(d, h, bytes) do { if ((bytes) > 0) { CHK(cuMemAlloc(&d, (bytes))); CHK(cuMemcpyHtoD(d, (h), (bytes))); } } while (0)
    ALLOC_COPY(d_pos, pos, b3);
    ALLOC_COPY(d_vel, vel, b3);
    ALLOC_COPY(d_mass, mass, sizeof(float) * (size_t)N);
    ALLOC_COPY(d_tris, tris, sizeof(int) * 3 * (size_t)T);
    ALLOC_COPY(d_G, Dm_inv, sizeof(float) * 4 * (size_t)T);
    ALLOC_COPY(d_area, rest_area, sizeof(float) * (size_t)T);
    ALLOC_COPY(d_k, stretch_k, sizeof(float) * (size_t)T);
    ALLOC_COPY(d_diag, diag, sizeof(float) * (size_t)N);
    ALLOC_COPY(d_quads, quads, sizeof(int) * 4 * (size_t)E);
    ALLOC_COPY(d_bw, bw, sizeof(float) * 4 * (size_t)E);
    ALLOC_COPY(d_bn, bn, sizeof(float) * (size_t)E);
    ALLOC_COPY(d_bk, bk, sizeof(float) * (size_t)E);
    ALLOC_COPY(d_pins, pins, sizeof(int) * (size_t)P);
    ALLOC_COPY(d_tgt, targets, sizeof(float) * 3 * (size_t)P);
    CHK(cuMemAlloc(&d_pred, b3));
    CHK(cuMemAlloc(&d_rhs, b3));
    CHK(cuMemAlloc(&d_prev, b3));
    CHK(cuMemAlloc(&d_new, b3));
    if (T > 0) CHK(cuMemAlloc(&d_proj, sizeof(float) * 6 * (size_t)T));
    if (E > 0) CHK(cuMemAlloc(&d_bproj, sizeof(float) * 3 * (size_t)E));

    {
        const float h2 = dt * dt;
        CHK(cuMemcpyDtoD(d_prev, d_pos, b3));
        { void* a[] = {&d_pos, &d_vel, &d_pred, &N, &dt, &gravity};
          CHK(cuLaunchKernel(fn[K_PREDICT], nb(N), 1, 1, 256, 1, 1, 0, 0, a, NULL)); }
        CUdeviceptr d_in = d_pos, d_out = d_new;
        for (int it = 0; it < iters; ++it) {
            if (T > 0) {
                void* a[] = {&d_in, &d_tris, &d_G, &d_proj, &T};
                CHK(cuLaunchKernel(fn[K_TRI], nb(T), 1, 1, 256, 1, 1, 0, 0, a, NULL));
            }
            if (E > 0) {
                void* a[] = {&d_in, &d_quads, &d_bw, &d_bn, &d_bproj, &E};
                CHK(cuLaunchKernel(fn[K_BEND], nb(E), 1, 1, 256, 1, 1, 0, 0, a, NULL));
            }
            { void* a[] = {&d_rhs, &N};
              CHK(cuLaunchKernel(fn[K_CLEAR], nb(N), 1, 1, 256, 1, 1, 0, 0, a, NULL)); }
            if (T > 0) {
                void* a[] = {&d_tris, &d_G, &d_area, &d_k, &d_proj, &d_rhs, &T, (void*)&h2};
                CHK(cuLaunchKernel(fn[K_TRI_RHS], nb(T), 1, 1, 256, 1, 1, 0, 0, a, NULL));
            }
            if (E > 0) {
                void* a[] = {&d_quads, &d_bw, &d_bk, &d_bproj, &d_rhs, &E, (void*)&h2};
                CHK(cuLaunchKernel(fn[K_BEND_RHS], nb(E), 1, 1, 256, 1, 1, 0, 0, a, NULL));
            }
            { void* a[] = {&d_rhs, &d_mass, &d_pred, &N};
              CHK(cuLaunchKernel(fn[K_INERT], nb(N), 1, 1, 256, 1, 1, 0, 0, a, NULL)); }
            { void* a[] = {&d_out, &d_rhs, &d_diag, &N};
              CHK(cuLaunchKernel(fn[K_DIV], nb(N), 1, 1, 256, 1, 1, 0, 0, a, NULL)); }
            if (P > 0) {
                void* a[] = {&d_out, &d_vel, &d_pins, &d_tgt, &P};
                CHK(cuLaunchKernel(fn[K_PINS], nb(P), 1, 1, 256, 1, 1, 0, 0, a, NULL));
            }
            { CUdeviceptr t = d_in; d_in = d_out; d_out = t; }
        }
        if (d_in != d_pos) CHK(cuMemcpyDtoD(d_pos, d_in, b3));
        { void* a[] = {&d_prev, &d_vel, &d_pos, &N, &dt, &damping};
          CHK(cuLaunchKernel(fn[K_VEL], nb(N), 1, 1, 256, 1, 1, 0, 0, a, NULL)); }
        if (P > 0) {
            void* a[] = {&d_pos, &d_vel, &d_pins, &d_tgt, &P};
            CHK(cuLaunchKernel(fn[K_PINS], nb(P), 1, 1, 256, 1, 1, 0, 0, a, NULL));
        }
        CHK(cuCtxSynchronize());
        CHK(cuMemcpyDtoH(pos, d_pos, b3));
        CHK(cuMemcpyDtoH(vel, d_vel, b3));
    }
done:
    {
        CUdeviceptr all[] = {d_pos, d_vel, d_mass, d_tris, d_G, d_area, d_k, d_diag, d_quads, d_bw, d_bn, d_bk,
                             d_pins, d_tgt, d_pred, d_rhs, d_prev, d_new, d_proj, d_bproj};
        for (size_t i = 0; i < sizeof(all) / sizeof(all[0]); ++i)
            if (all[i]) cuMemFree(all[i]);
    }
    if (mod) cuModuleUnload(mod);
    if (ctx) cuDevicePrimaryCtxRelease(dev);
    return rc;
}
