// Persistent whole-frame PD kernel: one cooperative launch runs predict, every
// sweep and the finalize of a frame, with a grid barrier between phases.
// Blocks loop over patches (patch = blockIdx.x + j * gridDim.x).  Every
// barrier wait is bounded by a clock64 budget: on expiry the block records
// an error code, and every block leaves the kernel at its next barrier, so no
// wait can hang the device.
#include "pd_kernels.cuh"
#include "pdg_kernels.h"

namespace pdg {

// Sense-free generation barrier over all blocks of a cooperative grid.
// bar[0] counts arrivals, bar[1] is the generation.  Returns false when this
// or any other block gave up waiting.
__device__ __forceinline__ bool grid_barrier(unsigned* bar, int* err, long long budget)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = bar + 1;
        const unsigned gen = *vgen;
        __threadfence();
        const unsigned arrived = atomicAdd(bar, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            const long long t0 = clock64();
            while (*vgen == gen) {
                if (clock64() - t0 > budget || *(volatile int*)err != 0) { atomicCAS(err, 0, 1); break; }
                __nanosleep(64);
            }
        }
        __threadfence();
        ok = (*(volatile int*)err == 0);
    }
    __syncthreads();
    return ok != 0;
}

template <int MODE, int NT>
__global__ void __launch_bounds__(NT) k_persistent(PersistArgs p)
{
    extern __shared__ float4 smem[];
    __shared__ PatchHdr ph;
    __shared__ float red[NT / 32];
    __shared__ int skip;
    __shared__ float omega;
    const IterArgs& a = p.it;
    const int gtid = blockIdx.x * NT + threadIdx.x, gstride = gridDim.x * NT;

    // predict + per-cloth reset
    for (int c = blockIdx.x; c < a.ncloth; c += gridDim.x) reset_rt(a.crt, a.acc, a.acc_stride, c, threadIdx.x, NT);
    for (int i = gtid; i < p.n; i += gstride)
        predict_vertex(i, p.X, p.V, p.aux, p.mass, p.vcloth, a.cinfo, p.warm, p.Y, a.buf[0], a.buf[1]);
    if (!grid_barrier(p.bar, p.err, p.spin_budget)) return;

    const int nsweep = p.max_iter + (p.have_final ? 1 : 0);
    for (int k = 0; k < nsweep; ++k) {
        const bool res_only = k >= p.max_iter;
        for (int pi = blockIdx.x; pi < p.npatch; pi += gridDim.x) {
            if (threadIdx.x == 0) {
                ph = a.patches[pi];
                const int c = ph.cloth;
                const ClothInfo& ci = a.cinfo[c];
                skip = cloth_done(a, c, k, pi == ci.patch_begin) ? 1 : 0;
                omega = (k < a.omega_stride) ? a.omega[c * a.omega_stride + k] : 1.f;
            }
            __syncthreads();
            if (!skip) {
                float4* sx = smem;
                float2* cxy = reinterpret_cast<float2*>(sx + 2 * ph.nlocal);
                float* cz = reinterpret_cast<float*>(cxy + ph.vm_nslot);
                process_patch<MODE, NT>(a, ph, k, res_only || k >= a.cinfo[ph.cloth].max_iter, omega,
                                        sx, cxy, cz, red);
            }
            __syncthreads();
        }
        if (!grid_barrier(p.bar, p.err, p.spin_budget)) return;
    }

    for (int c = gtid; c < a.ncloth; c += gstride) frame_stats_cloth(a, c);
    if (!grid_barrier(p.bar, p.err, p.spin_budget)) return;
    for (int i = gtid; i < p.n; i += gstride)
        finalize_vertex(i, p.Xw, p.V, p.Y, a.buf[0], a.buf[1], p.aux, p.vcloth, a.cinfo, a.crt);
}

template <int MODE, int NT>
static void* kernel_ptr() { return (void*)k_persistent<MODE, NT>; }

static void* pick(int mode, int nt)
{
    if (mode == kModeConsistent) {
        if (nt == 128) return kernel_ptr<kModeConsistent, 128>();
        if (nt == 256) return kernel_ptr<kModeConsistent, 256>();
        if (nt == 512) return kernel_ptr<kModeConsistent, 512>();
    } else {
        if (nt == 128) return kernel_ptr<kModeLiteral, 128>();
        if (nt == 256) return kernel_ptr<kModeLiteral, 256>();
        if (nt == 512) return kernel_ptr<kModeLiteral, 512>();
    }
    return nullptr;
}

int persistent_max_blocks(int mode, int nt, size_t smem, int* per_sm)
{
    void* f = pick(mode, nt);
    if (!f) return 0;
    if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) != cudaSuccess) return 0;
    int dev = 0, nsm = 0, nb = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, f, nt, smem) != cudaSuccess) return 0;
    if (per_sm) *per_sm = nb;
    return nb * nsm;
}

cudaError_t launch_persistent(const PersistArgs& p, int nt, int grid, size_t smem, cudaStream_t s)
{
    void* f = pick(p.mode, nt);
    if (!f || grid <= 0) return cudaErrorInvalidValue;
    PersistArgs copy = p;
    void* args[] = {&copy};
    return cudaLaunchCooperativeKernel(f, dim3(grid), dim3(nt), args, smem, s);
}

}  // namespace pdg
