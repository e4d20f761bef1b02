// pdg_step_noalloc: one frame of the consistent PD solve that allocates no
// device memory.
//
// Who needs it: callers that cannot call cudaMalloc -- applications that own
// all device memory through their own pool (engines and hosts that load this
// library as a plugin and forbid allocation behind their back), and real-time
// loops that cannot afford cudaMalloc/cudaFree, which synchronise the whole
// device.  They pass the cloth in the reference's own device layout (the
// arrays of ClothMesh, SimConstraints and Constraints) and get the frame
// solved in place.
//
// Where the scratch lives: the per-frame work arrays (inertial prediction,
// the two offset iterates, the force accumulator, the per-sweep residual
// sums and the control word) sit in one file-scope __device__ array of
// kScratchBytes (about 8.4 MB), which every GPU that loads the library holds
// until the process exits.  Sizes beyond PDG_NOALLOC_MAX_VERTS vertices or
// PDG_NOALLOC_MAX_ITERS sweeps are rejected.  Host code cannot use the
// array's name as a device address, so the first call on each device looks
// the address up with cudaGetSymbolAddress (with that device current) and
// caches it; make that first call before any stream capture.  All calls share
// the array and it keeps the last call's contents: each call clears what
// must start at zero, and calls that overlap on the GPU (different streams,
// or different host threads) race on it.
//
// The sweep structure is one launch per phase (clear, triangles, hinges,
// vertex update) with float atomics into the accumulator, so results match
// pdg_solver_step to rounding, not bitwise.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "../../include/pdg.h"
#include "pd_kernels.cuh"
#include "pdg_host.h"

namespace pdg {
namespace {

constexpr int kMaxVerts = PDG_NOALLOC_MAX_VERTS;
constexpr int kMaxIters = PDG_NOALLOC_MAX_ITERS;

struct NaCtl {
    int active, used, status, pad;
    double res_y2, res0_2, resf_2;
};

constexpr size_t kOffY = 0;
constexpr size_t kOffA = kOffY + 16 * (size_t)kMaxVerts;
constexpr size_t kOffB = kOffA + 16 * (size_t)kMaxVerts;
constexpr size_t kOffF = kOffB + 16 * (size_t)kMaxVerts;
constexpr size_t kOffAcc = kOffF + 16 * (size_t)kMaxVerts;
constexpr size_t kOffCtl = kOffAcc + 8 * (size_t)(kMaxIters + 2);
constexpr size_t kScratchBytes = kOffCtl + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct Scratch {
    float4* Y; float4* A; float4* B; float4* F; double* acc; NaCtl* ctl;
};

Scratch carve(unsigned char* base)
{
    Scratch s;
    s.Y = reinterpret_cast<float4*>(base + kOffY);
    s.A = reinterpret_cast<float4*>(base + kOffA);
    s.B = reinterpret_cast<float4*>(base + kOffB);
    s.F = reinterpret_cast<float4*>(base + kOffF);
    s.acc = reinterpret_cast<double*>(base + kOffAcc);
    s.ctl = reinterpret_cast<NaCtl*>(base + kOffCtl);
    return s;
}

inline int nb(int n, int b) { return (n + b - 1) / b; }

__global__ void k_na_setup(Scratch s, int nacc)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nacc) s.acc[i] = 0.0;
    if (i == 0) {
        NaCtl c;
        c.active = 1; c.used = 0; c.status = 0; c.pad = 0;
        c.res_y2 = 0.0; c.res0_2 = 0.0; c.resf_2 = -1.0;
        *s.ctl = c;
    }
}

__global__ void k_na_predict(Scratch s, int N, const float* __restrict__ pos, const float* __restrict__ vel,
                             const float* __restrict__ mass, const float* __restrict__ diag, float h, float ax,
                             float ay, float az)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const float h2 = fmul(h, h);
    float4 y;
    y.x = ffma(h2, ax, ffma(h, vel[3 * i], pos[3 * i]));
    y.y = ffma(h2, ay, ffma(h, vel[3 * i + 1], pos[3 * i + 1]));
    y.z = ffma(h2, az, ffma(h, vel[3 * i + 2], pos[3 * i + 2]));
    y.w = mass[i];
    s.Y[i] = y;
    const float dg = diag[i];
    const float4 d0 = make_float4(0.f, 0.f, 0.f, dg > 1e-10f ? 1.0f / dg : 0.f);   // inertial start
    s.A[i] = d0;
    s.B[i] = d0;
}

__global__ void k_na_pins(Scratch s, int P, const int* __restrict__ idx, const float* __restrict__ target)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= P) return;
    const int i = idx[q];
    const float4 y = s.Y[i];
    const float4 d = make_float4(fsub(target[3 * q], y.x), fsub(target[3 * q + 1], y.y), fsub(target[3 * q + 2], y.z), -1.f);
    s.A[i] = d;
    s.B[i] = d;
}

// Decision at the start of sweep k (same rules as the solver's per-cloth
// decision): converged, failed or capped frames become inactive.
__global__ void k_na_control(Scratch s, int k, int cap, float tol, int have_final)
{
    NaCtl& c = *s.ctl;
    if (!c.active) return;
    if (k >= 1) {
        const double acc0 = s.acc[0], rk2 = s.acc[k - 1];
        if (k == 1) { c.res0_2 = acc0; c.res_y2 = acc0; }
        if (!isfinite(rk2)) { c.status = -6; c.used = k - 1; c.resf_2 = rk2; c.active = 0; return; }
        if (tol > 0.f && rk2 <= (double)tol * (double)tol * c.res_y2) {
            c.used = k - 1; c.resf_2 = rk2; c.active = 0; return;
        }
    }
    if (k >= cap && !have_final) { c.used = cap; c.resf_2 = -1.0; c.active = 0; }
}

__global__ void k_na_clear(Scratch s, int N)
{
    if (!s.ctl->active) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < N) s.F[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

__device__ __forceinline__ void add3(float4* F, int v, float3 c)
{
    atomicAdd(&F[v].x, c.x); atomicAdd(&F[v].y, c.y); atomicAdd(&F[v].z, c.z);
}

__global__ void k_na_tri(Scratch s, int T, const int* __restrict__ tris, const float* __restrict__ Dm_inv,
                         const float* __restrict__ area, const float* __restrict__ ks, float h2, int k)
{
    if (!s.ctl->active) return;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    const float4* D = (k & 1) ? s.B : s.A;
    const int i0 = tris[3 * t], i1 = tris[3 * t + 1], i2 = tris[3 * t + 2];
    const float4 G = make_float4(Dm_inv[4 * t], Dm_inv[4 * t + 1], Dm_inv[4 * t + 2], Dm_inv[4 * t + 3]);
    float3 c0, c1, c2;
    tri_force<kModeConsistent>(edge(s.Y, D, i0, i1), edge(s.Y, D, i0, i2), G, h2 * (ks[t] * area[t]), c0, c1, c2);
    add3(s.F, i0, c0); add3(s.F, i1, c1); add3(s.F, i2, c2);
}

__global__ void k_na_hinge(Scratch s, int E, const int* __restrict__ quads, const float* __restrict__ w4,
                           const float* __restrict__ nrest, const float* __restrict__ kb, float h2, int k)
{
    if (!s.ctl->active) return;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const float4* D = (k & 1) ? s.B : s.A;
    const int i0 = quads[4 * e], i1 = quads[4 * e + 1], i2 = quads[4 * e + 2], i3 = quads[4 * e + 3];
    const float4 w = make_float4(w4[4 * e], w4[4 * e + 1], w4[4 * e + 2], w4[4 * e + 3]);
    const float4 y0 = s.Y[i0], d0 = D[i0];
    const float3 x0 = make_float3(fadd(y0.x, d0.x), fadd(y0.y, d0.y), fadd(y0.z, d0.z));
    const float3 q = hinge_force<kModeConsistent>(edge(s.Y, D, i0, i1), edge(s.Y, D, i0, i2), edge(s.Y, D, i0, i3),
                                                  x0, w, h2 * kb[e], nrest[e]);
    add3(s.F, i0, scale3(q, w.x)); add3(s.F, i1, scale3(q, w.y));
    add3(s.F, i2, scale3(q, w.z)); add3(s.F, i3, scale3(q, w.w));
}

__global__ void __launch_bounds__(256) k_na_update(Scratch s, int N, int k, int res_only, float omega, float gamma)
{
    __shared__ float red[8];
    if (!s.ctl->active) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const float4* Dk = (k & 1) ? s.B : s.A;
    float4* Dn = (k & 1) ? s.A : s.B;
    float r2 = 0.f;
    if (i < N) {
        const float4 d = Dk[i], y = s.Y[i], f4 = s.F[i];
        const float4 dp = res_only ? d : Dn[i];
        const float4 o = update_consistent(d, y, make_float3(f4.x, f4.y, f4.z), dp, gamma, omega, r2);
        if (!res_only) Dn[i] = o;
    }
    block_residual<256>(r2, red, s.acc + k);
}

__global__ void k_na_end(Scratch s, int cap, int have_final)
{
    NaCtl& c = *s.ctl;
    if (cap <= 1) { c.res0_2 = s.acc[0]; c.res_y2 = s.acc[0]; }
    if (!c.active) return;
    c.used = cap;
    bool finite = true;
    for (int k = 0; k <= cap; ++k) finite = finite && isfinite(s.acc[k]);
    c.resf_2 = have_final ? s.acc[cap] : -1.0;
    if (!finite) c.status = -6;
    c.active = 0;
}

__global__ void k_na_finalize(Scratch s, int N, float* __restrict__ pos, float* __restrict__ vel, float h,
                              float damping, float ax, float ay, float az)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const NaCtl c = *s.ctl;
    if (c.status != 0) {   // failed frame: keep x_n, stop the cloth
        vel[3 * i] = 0.f; vel[3 * i + 1] = 0.f; vel[3 * i + 2] = 0.f;
        return;
    }
    const float4 d = (c.used & 1) ? s.B[i] : s.A[i];
    const float4 y = s.Y[i];
    const float sc = 1.f - damping, ih = fdiv(1.f, h);
    vel[3 * i] = fmul(sc, ffma(d.x, ih, ffma(h, ax, vel[3 * i])));
    vel[3 * i + 1] = fmul(sc, ffma(d.y, ih, ffma(h, ay, vel[3 * i + 1])));
    vel[3 * i + 2] = fmul(sc, ffma(d.z, ih, ffma(h, az, vel[3 * i + 2])));
    pos[3 * i] = fadd(y.x, d.x); pos[3 * i + 1] = fadd(y.y, d.y); pos[3 * i + 2] = fadd(y.z, d.z);
}

__global__ void k_na_pins_final(int P, const int* __restrict__ idx, const float* __restrict__ target,
                                float* __restrict__ pos, float* __restrict__ vel)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= P) return;
    const int i = idx[q];
    pos[3 * i] = target[3 * q]; pos[3 * i + 1] = target[3 * q + 1]; pos[3 * i + 2] = target[3 * q + 2];
    vel[3 * i] = 0.f; vel[3 * i + 1] = 0.f; vel[3 * i + 2] = 0.f;
}

// Device address of the scratch array, looked up once per device.
std::mutex g_mu;
unsigned char* g_addr[64] = {};

int scratch_of(int dev, unsigned char** out)
{
    if (dev < 0 || dev >= 64) return set_error(PDG_ERR_ARG, "pdg_step_noalloc: device %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return set_error(PDG_ERR_CUDA, "pdg_step_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
        g_addr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_addr[dev];
    return PDG_OK;
}

}  // namespace
}  // namespace pdg

using namespace pdg;

#define NA_CK(call)                                                                                \
    do {                                                                                           \
        const cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) return set_error(PDG_ERR_CUDA, "pdg_step_noalloc: %s", cudaGetErrorString(e_)); \
    } while (0)

extern "C" int pdg_step_noalloc(const pdg_config* cfg, int N, float* d_pos, float* d_vel, const float* d_mass,
                                const float* d_jacobi_diag, int T, const int* d_tris, const float* d_Dm_inv,
                                const float* d_rest_area, const float* d_stretch_k, int E, const int* d_bend_quads,
                                const float* d_bend_w, const float* d_bend_n, const float* d_bend_k, int P,
                                const int* d_pin_idx, const float* d_pin_target, void* stream,
                                pdg_frame_stats* stats)
{
    if (!cfg) return set_error(PDG_ERR_ARG, "pdg_step_noalloc: null config");
    if (N <= 0 || N > kMaxVerts)
        return set_error(PDG_ERR_ARG, "pdg_step_noalloc: %d vertices; this entry point handles 1..%d", N, kMaxVerts);
    if (cfg->max_iterations < 0 || cfg->max_iterations > kMaxIters)
        return set_error(PDG_ERR_ARG, "pdg_step_noalloc: max_iterations %d; this entry point handles 0..%d",
                         cfg->max_iterations, kMaxIters);
    if (T < 0 || E < 0 || P < 0) return set_error(PDG_ERR_ARG, "pdg_step_noalloc: negative count");
    if (cfg->mode != PDG_MODE_CONSISTENT || cfg->init != PDG_INIT_INERTIAL)
        return set_error(PDG_ERR_ARG, "pdg_step_noalloc: only the consistent mode from the inertial start");
    if (!(cfg->dt > 0.f) || !(cfg->damping >= 0.f && cfg->damping <= 1.f) || !(cfg->gamma > 0.f) ||
        (cfg->use_chebyshev && !(cfg->rho >= 0.f && cfg->rho < 1.f)) || cfg->cheb_delay < 0)
        return set_error(PDG_ERR_ARG, "pdg_step_noalloc: invalid dt, damping, gamma, rho or cheb_delay");
    if (!d_pos || !d_vel || !d_mass || !d_jacobi_diag || (T && (!d_tris || !d_Dm_inv || !d_rest_area || !d_stretch_k)) ||
        (E && (!d_bend_quads || !d_bend_w || !d_bend_n || !d_bend_k)) || (P && (!d_pin_idx || !d_pin_target)))
        return set_error(PDG_ERR_ARG, "pdg_step_noalloc: null device array");

    int dev = 0;
    NA_CK(cudaGetDevice(&dev));
    if (stream) {   // the scratch address is this device's: the stream must belong to it
        int sdev = -1;
        NA_CK(cudaStreamGetDevice(static_cast<cudaStream_t>(stream), &sdev));
        if (sdev != dev)
            return set_error(PDG_ERR_ARG, "pdg_step_noalloc: the stream belongs to device %d, the current device is %d",
                             sdev, dev);
    }
    unsigned char* base = nullptr;
    const int rc = scratch_of(dev, &base);
    if (rc) return rc;
    const Scratch s = carve(base);
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    const int cap = cfg->max_iterations;
    const int have_final = (cfg->compute_final_residual || cfg->tolerance > 0.f) ? 1 : 0;
    const float h = cfg->dt, h2 = h * h;
    const float ax = cfg->wind[0], ay = cfg->gravity + cfg->wind[1], az = cfg->wind[2];

    k_na_setup<<<nb(cap + 2, 256), 256, 0, st>>>(s, cap + 2);
    k_na_predict<<<nb(N, 256), 256, 0, st>>>(s, N, d_pos, d_vel, d_mass, d_jacobi_diag, h, ax, ay, az);
    if (P) k_na_pins<<<nb(P, 128), 128, 0, st>>>(s, P, d_pin_idx, d_pin_target);
    float om = 1.f;
    const float r2 = cfg->rho * cfg->rho;
    const int nsweep = cap + have_final;
    for (int k = 0; k < nsweep; ++k) {
        const bool res_only = k >= cap;
        if (!res_only) {   // Chebyshev weight of sweep k (same recurrence as the solver)
            if (!cfg->use_chebyshev || k < cfg->cheb_delay) om = 1.f;
            else if (k == cfg->cheb_delay) om = 2.f / (2.f - r2);
            else om = 4.f / (4.f - r2 * om);
        }
        k_na_control<<<1, 1, 0, st>>>(s, k, cap, cfg->tolerance, have_final);
        k_na_clear<<<nb(N, 256), 256, 0, st>>>(s, N);
        if (T) k_na_tri<<<nb(T, 256), 256, 0, st>>>(s, T, d_tris, d_Dm_inv, d_rest_area, d_stretch_k, h2, k);
        if (E) k_na_hinge<<<nb(E, 256), 256, 0, st>>>(s, E, d_bend_quads, d_bend_w, d_bend_n, d_bend_k, h2, k);
        k_na_update<<<nb(N, 256), 256, 0, st>>>(s, N, k, res_only ? 1 : 0, res_only ? 1.f : om, cfg->gamma);
    }
    k_na_end<<<1, 1, 0, st>>>(s, cap, have_final);
    k_na_finalize<<<nb(N, 256), 256, 0, st>>>(s, N, d_pos, d_vel, h, cfg->damping, ax, ay, az);
    if (P) k_na_pins_final<<<nb(P, 128), 128, 0, st>>>(P, d_pin_idx, d_pin_target, d_pos, d_vel);
    NA_CK(cudaGetLastError());

    if (stats) {
        NaCtl c;
        NA_CK(cudaMemcpyAsync(&c, s.ctl, sizeof(NaCtl), cudaMemcpyDeviceToHost, st));
        NA_CK(cudaStreamSynchronize(st));
        stats->iterations = c.used;
        stats->warm_start_used = 0;
        stats->status = c.status;
        stats->res_inertial = std::sqrt(std::fmax(0.0, c.res_y2));
        stats->res_initial = std::sqrt(std::fmax(0.0, c.res0_2));
        stats->res_final = c.resf_2 >= 0.0 ? std::sqrt(c.resf_2) : -1.0;
        stats->rel_residual = (stats->res_final >= 0.0 && stats->res_inertial > 0.0)
                                  ? stats->res_final / stats->res_inertial : -1.0;
        stats->converged = (c.status == 0 && cfg->tolerance > 0.f && stats->res_final >= 0.0 &&
                            stats->res_final <= (double)cfg->tolerance * stats->res_inertial) ? 1 : 0;
    }
    return PDG_OK;
}
