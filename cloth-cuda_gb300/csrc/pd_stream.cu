// Streaming sweep: one launch per Jacobi sweep (replayed from the frame's CUDA
// graph) with a persistent grid of a few blocks per SM.  Each block walks the
// patches blockIdx.x, blockIdx.x + gridDim.x, ... and double-buffers them in
// shared memory: while it projects and gathers patch i, the TMA engine copies
// the contiguous per-patch data of patch i + gridDim.x (cell and lone hinge
// records, gather pointers and entries, halo index list, y, d^k and d^(k-1)
// of the owned vertices) into the other stage with cp.async.bulk, completing
// on an mbarrier.  Only the halo vertices' y and d^k are gathered with plain
// loads.  The per-vertex arithmetic is the one of the per-patch sweep
// (same device functions, same slot order), so the results are bitwise equal.
//
// Every mbarrier wait is bounded by a clock64 budget.  On expiry the block
// records an error code, waits (bounded) for its copies still in flight and
// leaves; the host reports PDG_ERR_TIMEOUT.
#include <cstdint>

#include "pd_kernels.cuh"
#include "pdg_kernels.h"

namespace pdg {

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Bounded wait for the phase with the given parity to complete: one
// non-blocking probe, then try_wait (which may suspend the thread for a
// while in hardware) until the clock64 budget is spent.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long budget)
{
    if (mbar_test_wait(bar, parity)) return true;
    const long long t0 = clock64();
    for (;;) {
        if (clock64() - t0 > budget) return false;
        if (mbar_try_wait(bar, parity)) return true;
    }
}

// Order this thread's earlier generic-proxy accesses of shared memory before
// later async-proxy (TMA) writes to it.
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Bulk copy global -> shared (both 16-byte aligned, bytes a multiple of 16),
// completing `bytes` transactions on `bar`.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ uint32_t round16(uint32_t b) { return (b + 15u) & ~15u; }

// Thread 0: header of patch p into *hs, then every contiguous list of the
// patch into `stage`, completing on `bar`.
__device__ __forceinline__ void issue_patch(const IterArgs& a, const StreamArgs& sa, const float4* Dk,
                                            const float4* Dn, int p, PatchHdr* hs, unsigned char* stage,
                                            uint64_t* bar)
{
    const PatchHdr h = a.patches[p];
    *hs = h;
    const uint32_t b_cell = (uint32_t)sizeof(CellRec) * h.ncell, b_hin = 32u * h.nhinge;
    const uint32_t b_ptr = round16(4u * (h.nown + 1)), b_ent = round16(2u * h.nent);
    const uint32_t b_hidx = round16(4u * (h.nlocal - h.nown)), b_v = 16u * h.nown;
    mbar_arrive_expect_tx(bar, b_cell + b_hin + b_ptr + b_ent + b_hidx + 3 * b_v);
    if (b_cell) bulk_g2s(stage + sa.o_cell, a.cells + h.cell_off, b_cell, bar);
    if (b_hin) bulk_g2s(stage + sa.o_hin, a.hinges + h.hinge_off, b_hin, bar);
    bulk_g2s(stage + sa.o_ptr, a.csr_ptr + h.csr_off, b_ptr, bar);
    if (b_ent) bulk_g2s(stage + sa.o_ent, a.csr_ent + h.ent_off, b_ent, bar);
    if (b_hidx) bulk_g2s(stage + sa.o_hidx, a.halo + h.halo_off, b_hidx, bar);
    if (b_v) {
        bulk_g2s(stage + sa.o_y, a.Y + h.vbegin, b_v, bar);
        bulk_g2s(stage + sa.o_d, Dk + h.vbegin, b_v, bar);
        bulk_g2s(stage + sa.o_dp, Dn + h.vbegin, b_v, bar);
    }
}

template <int MODE, int NT>
__global__ void __launch_bounds__(NT) k_stream(IterArgs a, StreamArgs sa, int k, int res_only)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ PatchHdr ph[2];
    __shared__ float red[NT / 32];
    __shared__ int skip;
    __shared__ float omega;
    const int tid = threadIdx.x;
    const float4* __restrict__ Dk = (k & 1) ? a.buf[1] : a.buf[0];
    float4* __restrict__ Dn = (k & 1) ? a.buf[0] : a.buf[1];
    float* cx = reinterpret_cast<float*>(smem_raw + sa.slot_off);
    float* cy = cx + sa.max_nslot;
    float* cz = cy + sa.max_nslot;

    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_fence_init();
    }
    __syncthreads();
    if (tid == 0 && (int)blockIdx.x < sa.npatch)
        issue_patch(a, sa, Dk, Dn, blockIdx.x, &ph[0], smem_raw, &bar[0]);

    uint32_t parity = 0;   // bit s: parity of the next phase of bar[s]
    int it = 0;
    for (int p = blockIdx.x; p < sa.npatch; p += gridDim.x, ++it) {
        const int s = it & 1;
        unsigned char* st = smem_raw + s * sa.stage_bytes;
        const bool got = mbar_wait(&bar[s], (parity >> s) & 1u, sa.spin_budget);
        parity ^= 1u << s;
        const bool has_next = p + (int)gridDim.x < sa.npatch;
        if (!__syncthreads_and(got)) {
            // give up: record the error, let copies in flight land, leave
            if (tid == 0) {
                atomicCAS(sa.err, 0, 4);
                // the drain has its own budget (about 2 s): the copies are
                // bounded in size and land unless the memory system failed
                if (!got) mbar_wait(&bar[s], ((parity >> s) & 1u) ^ 1u, 4000000000LL);
            }
            __syncthreads();
            return;
        }
        if (tid == 0) {
            if (has_next) {   // stage s^1 was released by the sync that ended the previous patch
                fence_proxy_async_smem();
                issue_patch(a, sa, Dk, Dn, p + gridDim.x, &ph[s ^ 1], smem_raw + (s ^ 1) * sa.stage_bytes,
                            &bar[s ^ 1]);
            }
            const PatchHdr& h = ph[s];
            const ClothInfo& ci = a.cinfo[h.cloth];
            skip = cloth_done(a, h.cloth, k, p == ci.patch_begin) ? 1 : 0;
            omega = (k < a.omega_stride) ? a.omega[h.cloth * a.omega_stride + k] : 1.f;
        }
        const PatchHdr& h = ph[s];
        const int nown = h.nown, nlocal = h.nlocal;
        float4* sy = reinterpret_cast<float4*>(st + sa.o_y);
        float4* sd = reinterpret_cast<float4*>(st + sa.o_d);
        const int* hidx = reinterpret_cast<const int*>(st + sa.o_hidx);
        for (int l = nown + tid; l < nlocal; l += NT) {
            const int g = hidx[l - nown];
            sy[l] = __ldcg(&a.Y[g]);
            sd[l] = __ldcg(&Dk[g]);
        }
        __syncthreads();
        if (!skip) {
            const int ncell = h.ncell, nhin = h.nhinge;
            const CellRec* cr = reinterpret_cast<const CellRec*>(st + sa.o_cell);
            const HingeRec* hr = reinterpret_cast<const HingeRec*>(st + sa.o_hin);
            for (int c = tid; c < ncell; c += NT) cell_contrib<MODE>(cr[c], sy, sd, c, ncell, cx, cy, cz);
            for (int e = tid; e < nhin; e += NT) hinge_contrib<MODE>(hr[e], sy, sd, e, 6 * ncell, nhin, cx, cy, cz);
            __syncthreads();
            const bool ro = res_only != 0 || k >= a.cinfo[h.cloth].max_iter;
            const float gamma = a.cinfo[h.cloth].gamma;
            const int* cp = reinterpret_cast<const int*>(st + sa.o_ptr);
            const uint16_t* ce = reinterpret_cast<const uint16_t*>(st + sa.o_ent);
            const float4* sdp = reinterpret_cast<const float4*>(st + sa.o_dp);
            float r2 = 0.f;
            for (int l = tid; l < nown; l += NT) {
                const float3 f = gather_force(ce, cp[l], cp[l + 1], cx, cy, cz);
                const int g = h.vbegin + l;
                const float4 d = sd[l];
                const float4 y = sy[l];
                if (MODE == kModeConsistent) {
                    float rv;
                    const float4 dp = ro ? d : sdp[l];
                    const float4 o = update_consistent(d, y, f, dp, gamma, omega, rv);
                    r2 += rv;
                    if (!ro) Dn[g] = o;
                } else if (!ro) {
                    Dn[g] = update_literal(d, y, f);
                }
            }
            if (MODE == kModeConsistent) block_residual<NT>(r2, red, a.acc + (size_t)h.cloth * a.acc_stride + k);
        }
        __syncthreads();   // stage s, the slots and the header are free again
    }
}

// Stage layout: every region starts on a 16-byte boundary.
bool stream_layout(int max_ncell, int max_nhinge, int max_nown, int max_nent, int max_nhalo, int max_nlocal,
                   int max_nslot, StreamArgs& sa, size_t& smem)
{
    auto r16 = [](size_t b) { return (b + 15) / 16 * 16; };
    size_t o = 0;
    sa.o_cell = (int)o; o += sizeof(CellRec) * (size_t)max_ncell;
    sa.o_hin = (int)o;  o += 32 * (size_t)max_nhinge;
    sa.o_ptr = (int)o;  o += r16(4 * (size_t)(max_nown + 1));
    sa.o_ent = (int)o;  o += r16(2 * (size_t)max_nent);
    sa.o_hidx = (int)o; o += r16(4 * (size_t)max_nhalo);
    sa.o_y = (int)o;    o += 16 * (size_t)max_nlocal;
    sa.o_d = (int)o;    o += 16 * (size_t)max_nlocal;
    sa.o_dp = (int)o;   o += 16 * (size_t)max_nown;
    o = (o + 127) / 128 * 128;
    sa.stage_bytes = (int)o;
    sa.slot_off = (int)(2 * o);
    sa.max_nslot = max_nslot;
    smem = 2 * o + 12 * (size_t)max_nslot;
    return smem < (1u << 31);
}

template <int MODE, int NT>
static void* stream_ptr() { return (void*)k_stream<MODE, NT>; }

static void* pick_stream(int mode, int nt)
{
    if (mode == kModeConsistent) {
        if (nt == 128) return stream_ptr<kModeConsistent, 128>();
        if (nt == 256) return stream_ptr<kModeConsistent, 256>();
        if (nt == 512) return stream_ptr<kModeConsistent, 512>();
    } else {
        if (nt == 128) return stream_ptr<kModeLiteral, 128>();
        if (nt == 256) return stream_ptr<kModeLiteral, 256>();
        if (nt == 512) return stream_ptr<kModeLiteral, 512>();
    }
    return nullptr;
}

int stream_max_blocks(int mode, int nt, size_t smem)
{
    void* f = pick_stream(mode, nt);
    if (!f) return 0;
    int dev = 0, nsm = 0, optin = 0, nb = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
    if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - 1024) != cudaSuccess) return 0;
    if (smem > (size_t)(optin - 1024)) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, f, nt, smem) != cudaSuccess) return 0;
    return nb * nsm;
}

cudaError_t launch_stream(const IterArgs& a, const StreamArgs& sa, int mode, int nt, int grid, size_t smem, int k,
                          int res_only, cudaStream_t s)
{
    void* f = pick_stream(mode, nt);
    if (!f || grid <= 0) return cudaErrorInvalidValue;
    IterArgs ac = a;
    StreamArgs sc = sa;
    void* args[] = {&ac, &sc, &k, &res_only};
    return cudaLaunchKernel(f, dim3(grid), dim3(nt), args, smem, s);
}

}  // namespace pdg
