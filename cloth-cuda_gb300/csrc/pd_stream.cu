// Streaming sweep: one launch per Jacobi sweep (replayed from the frame's CUDA
// graph) on a persistent grid of resident blocks.  Block b walks the patches
// b, b + G, b + 2G, ... (G = grid size) and software-pipelines their staging
// so that the memory round trips of patch p + G overlap the arithmetic of
// patch p:
//   - the TMA engine bulk-copies p + G's contiguous lists (halo index list,
//     gather pointers, y, d^k and d^(k-1) of the owned vertices) into the
//     other of two stages while the block projects patch p's cells;
//   - after p's cell step every thread gathers p + G's halo y and d^k into
//     that stage with asynchronous 16-byte copies (cp.async), which land
//     while the block gathers patch p's contributions;
//   - the header of p + 2G is copied into a three-entry ring, and the
//     per-cloth decision for p + G is taken one patch ahead.
// Cell and hinge records are read from global memory as in the per-patch
// sweep, so a stage holds only vertex data and several blocks fit per SM.
// The per-vertex arithmetic, the vertex-major slots and the gather order are
// those of the per-patch sweep (same device functions), so the results are
// bitwise equal.
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

// Per-thread asynchronous 16-byte copy global -> shared (cached in L2 only),
// tracked by the thread's cp.async groups.
__device__ __forceinline__ void cp_async16(void* dst, const void* src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)),
                 "l"(__cvta_generic_to_global(src))
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Bulk prefetch into L2 of the 16-byte-aligned part of [p, p + bytes).
__device__ __forceinline__ void prefetch_l2(const void* p, size_t bytes)
{
    const size_t g = __cvta_generic_to_global(p);
    const size_t b = (g + 15) & ~(size_t)15;
    const size_t e = (g + bytes) & ~(size_t)15;
    if (e > b) asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(b), "r"((unsigned)(e - b)) : "memory");
}

// Thread 0: every contiguous list of patch h into `stage`, completing on
// `bar`; the patch's cell records are started towards L2.
__device__ __forceinline__ void issue_patch(const IterArgs& a, const StreamArgs& sa, const float4* Dk,
                                            const float4* Dn, const PatchHdr& h, unsigned char* stage,
                                            uint64_t* bar)
{
    const uint32_t b_ptr = round16(4u * (h.nown + 1));
    const uint32_t b_hidx = round16(4u * (h.nlocal - h.nown)), b_v = 16u * h.nown;
    mbar_arrive_expect_tx(bar, b_ptr + b_hidx + 3 * b_v);
    bulk_g2s(stage + sa.o_ptr, a.csr_ptr + h.csr_off, b_ptr, bar);
    if (b_hidx) bulk_g2s(stage + sa.o_hidx, a.halo + h.halo_off, b_hidx, bar);
    if (b_v) {
        bulk_g2s(stage + sa.o_y, a.Y + h.vbegin, b_v, bar);
        bulk_g2s(stage + sa.o_d, Dk + h.vbegin, b_v, bar);
        bulk_g2s(stage + sa.o_dp, Dn + h.vbegin, b_v, bar);
    }
    prefetch_l2(a.cells + h.cell_off, sizeof(CellRec) * (size_t)((h.ncell + kCellGroup - 1) / kCellGroup * kCellGroup));
}

// Thread 0: asynchronous copy of a patch header (80 bytes, 16-byte aligned
// in both spaces) into the header ring.
__device__ __forceinline__ void copy_header(const PatchHdr* src, PatchHdr* dst)
{
    static_assert(sizeof(PatchHdr) % 16 == 0, "PatchHdr is copied in 16-byte pieces");
    #pragma unroll
    for (int i = 0; i < (int)(sizeof(PatchHdr) / 16); ++i)
        cp_async16(reinterpret_cast<unsigned char*>(dst) + 16 * i, reinterpret_cast<const unsigned char*>(src) + 16 * i);
}

// Per-patch decision, taken by one thread one patch ahead.
struct PatchDecision {
    int   skip;    // cloth done: nothing to compute
    int   ro;      // residual only (no update)
    float omega;   // Chebyshev weight of this sweep
    float gamma;   // under-relaxation
};

__device__ __forceinline__ void decide(const IterArgs& a, const PatchHdr& h, int p, int k, int res_only,
                                       PatchDecision* out)
{
    const int c = h.cloth;
    const ClothInfo& ci = a.cinfo[c];
    PatchDecision d;
    d.skip = cloth_done(a, c, k, p == ci.patch_begin) ? 1 : 0;
    d.ro = (res_only != 0 || k >= ci.max_iter) ? 1 : 0;
    d.omega = (k < a.omega_stride) ? a.omega[c * a.omega_stride + k] : 1.f;
    d.gamma = ci.gamma;
    *out = d;
}

// Programmatic dependent launch: wait until the grids this one depends on
// have completed and their memory is visible (returns at once without
// such a dependency), and allow the dependent grid to be scheduled.
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_dep_launch_dependents()
{
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Thread 0, first patch only: the lists of patch h that the previous sweep
// does not write (halo index list, gather pointers, y and d^(k-1) of the
// owned vertices) into `stage`, completing on `bar`.
__device__ __forceinline__ void issue_static(const IterArgs& a, const StreamArgs& sa, const float4* Dn,
                                             const PatchHdr& h, unsigned char* stage, uint64_t* bar)
{
    const uint32_t b_ptr = round16(4u * (h.nown + 1));
    const uint32_t b_hidx = round16(4u * (h.nlocal - h.nown)), b_v = 16u * h.nown;
    mbar_arrive_expect_tx(bar, b_ptr + b_hidx + 2 * b_v);
    bulk_g2s(stage + sa.o_ptr, a.csr_ptr + h.csr_off, b_ptr, bar);
    if (b_hidx) bulk_g2s(stage + sa.o_hidx, a.halo + h.halo_off, b_hidx, bar);
    if (b_v) {
        bulk_g2s(stage + sa.o_y, a.Y + h.vbegin, b_v, bar);
        bulk_g2s(stage + sa.o_dp, Dn + h.vbegin, b_v, bar);
    }
    prefetch_l2(a.cells + h.cell_off, sizeof(CellRec) * (size_t)((h.ncell + kCellGroup - 1) / kCellGroup * kCellGroup));
}

// Thread 0, first patch only: d^k of the owned vertices, completing on `bar`.
__device__ __forceinline__ void issue_dk(const StreamArgs& sa, const float4* Dk, const PatchHdr& h,
                                         unsigned char* stage, uint64_t* bar)
{
    const uint32_t b_v = 16u * h.nown;
    mbar_arrive_expect_tx(bar, b_v);
    if (b_v) bulk_g2s(stage + sa.o_d, Dk + h.vbegin, b_v, bar);
}

// Every thread, first patch only: its share of the halo y, then of the halo
// d^k (after the previous sweep completed), into `stage`.
__device__ __forceinline__ void gather_halo_y(const IterArgs& a, const StreamArgs& sa, const PatchHdr& h,
                                              unsigned char* stage, int tid, int nt)
{
    const int* hidx = reinterpret_cast<const int*>(stage + sa.o_hidx);
    float4* sy = reinterpret_cast<float4*>(stage + sa.o_y);
    for (int l = h.nown + tid; l < h.nlocal; l += nt) cp_async16(&sy[l], &a.Y[hidx[l - h.nown]]);
}
__device__ __forceinline__ void gather_halo_d(const StreamArgs& sa, const float4* Dk, const PatchHdr& h,
                                              unsigned char* stage, int tid, int nt)
{
    const int* hidx = reinterpret_cast<const int*>(stage + sa.o_hidx);
    float4* sd = reinterpret_cast<float4*>(stage + sa.o_d);
    for (int l = h.nown + tid; l < h.nlocal; l += nt) cp_async16(&sd[l], &Dk[hidx[l - h.nown]]);
    cp_async_commit();
}

// Every thread: its share of patch h's halo y and d^k into `stage`.
__device__ __forceinline__ void gather_halo(const IterArgs& a, const StreamArgs& sa, const float4* Dk,
                                            const PatchHdr& h, unsigned char* stage, int tid, int nt)
{
    const int* hidx = reinterpret_cast<const int*>(stage + sa.o_hidx);
    float4* sy = reinterpret_cast<float4*>(stage + sa.o_y);
    float4* sd = reinterpret_cast<float4*>(stage + sa.o_d);
    const int nown = h.nown, nlocal = h.nlocal;
    for (int l = nown + tid; l < nlocal; l += nt) {
        const int g = hidx[l - nown];
        cp_async16(&sy[l], &a.Y[g]);
        cp_async16(&sd[l], &Dk[g]);
    }
    cp_async_commit();
}

// The register cap is set for 6 blocks of 128 threads per SM (80 registers,
// no spills); measured on 1025x1025 and the 512-cloth batch it is about 1 %
// faster than the cap for 5 (96 registers).
template <int MODE, int NT>
__global__ void __launch_bounds__(NT, 768 / NT) k_stream(IterArgs a, StreamArgs sa, int k, int res_only)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar[3];   // the two stages; the first patch's static lists
    __shared__ __align__(16) PatchHdr hring[3];
    __shared__ PatchDecision dec[2];
    __shared__ float red[NT / 32];
    const int tid = threadIdx.x;
    const int G = gridDim.x;
    const float4* __restrict__ Dk = (k & 1) ? a.buf[1] : a.buf[0];
    float4* __restrict__ Dn = (k & 1) ? a.buf[0] : a.buf[1];
    float2* cxy = reinterpret_cast<float2*>(smem_raw + sa.slot_off);
    float* cz = reinterpret_cast<float*>(cxy + sa.max_nslot);
    const int p0 = blockIdx.x;
    if (p0 >= sa.npatch) return;

    // Prologue.  Launched as a programmatic dependent of the previous sweep,
    // the block may start while that sweep's last blocks still run.  Before
    // griddepcontrol.wait it reads only what no sweep of this frame writes
    // (patch headers, halo lists, gather pointers, y) or what the sweep
    // before the previous one wrote (d^(k-1)); it signals its own
    // dependents only after the wait, so when the next sweep's blocks start
    // early, the previous sweep has completed.  d^k, the per-sweep sums and
    // the runtime records are read after the wait.
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_init(&bar[2], 1);
        mbar_fence_init();
        hring[0] = a.patches[p0];
        if (p0 + G < sa.npatch) copy_header(a.patches + p0 + G, &hring[1]);
        cp_async_commit();
    }
    __syncthreads();
    if (tid == 0) issue_static(a, sa, Dn, hring[0], smem_raw, &bar[2]);
    {
        const bool got = mbar_wait(&bar[2], 0, sa.spin_budget);
        if (!__syncthreads_and(got)) {
            if (tid == 0) {
                atomicCAS(sa.err, 0, 4);
                if (!got) mbar_wait(&bar[2], 0, 4000000000LL);
            }
            cp_async_wait_all();
            __syncthreads();
            return;
        }
    }
    gather_halo_y(a, sa, hring[0], smem_raw, tid, NT);
    grid_dep_wait();
    grid_dep_launch_dependents();
    if (tid == 0) {
        issue_dk(sa, Dk, hring[0], smem_raw, &bar[0]);
        decide(a, hring[0], p0, k, res_only, &dec[0]);
    }
    gather_halo_d(sa, Dk, hring[0], smem_raw, tid, NT);
    uint32_t parity = 0;   // bit s: parity of the next phase of bar[s]
    {
        const bool got = mbar_wait(&bar[0], 0, sa.spin_budget);
        parity ^= 1u;
        if (!__syncthreads_and(got)) {
            if (tid == 0) {
                atomicCAS(sa.err, 0, 4);
                if (!got) mbar_wait(&bar[0], 0, 4000000000LL);
            }
            cp_async_wait_all();
            __syncthreads();
            return;
        }
    }

    int it = 0;
    for (int p = p0; p < sa.npatch; p += G, ++it) {
        const int s = it & 1;
        const int q = p + G;
        unsigned char* st = smem_raw + s * sa.stage_bytes;
        unsigned char* st1 = smem_raw + (s ^ 1) * sa.stage_bytes;
        // patch p's stage, header and decision are complete; the other stage
        // and the slots are free
        cp_async_wait_all();
        __syncthreads();
        const PatchHdr& h = hring[it % 3];
        if (tid == 0 && q < sa.npatch) {
            const PatchHdr& hq = hring[(it + 1) % 3];
            fence_proxy_async_smem();
            issue_patch(a, sa, Dk, Dn, hq, st1, &bar[s ^ 1]);
            if (q + G < sa.npatch) copy_header(a.patches + q + G, &hring[(it + 2) % 3]);
            cp_async_commit();
        }
        // the decision for q (one memory round trip) is taken by another
        // warp than the copy issue, so neither warp carries both
        if (tid == 32 && q < sa.npatch) decide(a, hring[(it + 1) % 3], q, k, res_only, &dec[s ^ 1]);
        const PatchDecision dp_ = dec[s];
        const float4* sy = reinterpret_cast<const float4*>(st + sa.o_y);
        const float4* sd = reinterpret_cast<const float4*>(st + sa.o_d);

        // local step of patch p: records from global memory, contributions
        // to the vertex-major slots.  Odd rounds run in reverse thread order,
        // so warps 0 and 1, which issue the copies and take the decision
        // above, get the lighter load.
        if (!dp_.skip) {
            const CellRec* __restrict__ cr = a.cells + h.cell_off;
            const int ncell = h.ncell, nhin = h.nhinge;
            for (int r = 0; r * NT < ncell; ++r) {
                const int c = r * NT + ((r & 1) ? NT - 1 - tid : tid);
                if (c < ncell) {
                    const CellRec rec = load_cell(cr, c);
                    cell_contrib_vm<MODE>(rec, const_cast<float4*>(sy), const_cast<float4*>(sd), cxy, cz);
                }
            }
            const HingeRec* __restrict__ hr = a.hinges + h.hinge_off;
            const uint2* __restrict__ hv = a.hvm + h.hinge_off;
            for (int e = tid; e < nhin; e += NT) {
                const HingeRec rec = hr[e];
                hinge_contrib_vm<MODE>(rec, __ldg(&hv[e]), const_cast<float4*>(sy), const_cast<float4*>(sd), cxy,
                                       cz);
            }
        }

        // patch q's lists have landed (or the wait gave up) and every
        // thread's contributions to p's slots are stored: one barrier
        const int b1 = s ^ 1;
        bool got = true;
        if (q < sa.npatch) {
            got = mbar_wait(&bar[b1], (parity >> b1) & 1u, sa.spin_budget);
            parity ^= 1u << b1;
        }
        if (!__syncthreads_and(got)) {
            // give up: record the error, let copies in flight land, leave
            if (tid == 0) {
                atomicCAS(sa.err, 0, 4);
                // the drain has its own budget (about 2 s): the copies are
                // bounded in size and land unless the memory system failed
                if (!got) mbar_wait(&bar[b1], ((parity >> b1) & 1u) ^ 1u, 4000000000LL);
            }
            cp_async_wait_all();
            __syncthreads();
            return;
        }
        // patch q's halo, gathered while patch p is finished
        if (q < sa.npatch) gather_halo(a, sa, Dk, hring[(it + 1) % 3], st1, tid, NT);

        // global step of patch p
        if (!dp_.skip) {
            const int nown = h.nown, vbegin = h.vbegin, npad = h.vm_npad;
            const int* cp = reinterpret_cast<const int*>(st + sa.o_ptr);
            const float4* sdp = reinterpret_cast<const float4*>(st + sa.o_dp);
            float r2 = 0.f;
            for (int l = tid; l < nown; l += NT) {
                const int deg = cp[l + 1] - cp[l];
                const int hh = gather_half(deg);
                const float3 f =
                    deg <= 10 ? fadd3(gather_vm_p<5>(l, 0, hh, npad, cxy, cz), gather_vm_p<5>(l, hh, deg, npad, cxy, cz))
                              : fadd3(gather_vm(l, 0, hh, npad, cxy, cz), gather_vm(l, hh, deg, npad, cxy, cz));
                const int g = vbegin + l;
                const float4 d = sd[l];
                const float4 y = sy[l];
                if (MODE == kModeConsistent) {
                    float rv;
                    const float4 dprev = dp_.ro ? d : sdp[l];
                    const float4 o = update_consistent(d, y, f, dprev, dp_.gamma, dp_.omega, rv);
                    r2 += rv;
                    if (!dp_.ro) Dn[g] = o;
                } else if (!dp_.ro) {
                    Dn[g] = update_literal(d, y, f);
                }
            }
            if (MODE == kModeConsistent) block_residual<NT>(r2, red, a.acc + (size_t)h.cloth * a.acc_stride + k);
        }
    }
    cp_async_wait_all();
}

// Stage layout: every region starts on a 16-byte boundary.
bool stream_layout(int max_nown, int max_nhalo, int max_nlocal, int max_vm_nslot, StreamArgs& sa, size_t& smem)
{
    auto r16 = [](size_t b) { return (b + 15) / 16 * 16; };
    size_t o = 0;
    sa.o_hidx = (int)o; o += r16(4 * (size_t)max_nhalo);
    sa.o_ptr = (int)o;  o += r16(4 * (size_t)(max_nown + 1));
    sa.o_y = (int)o;    o += 16 * (size_t)max_nlocal;
    sa.o_d = (int)o;    o += 16 * (size_t)max_nlocal;
    sa.o_dp = (int)o;   o += 16 * (size_t)max_nown;
    o = (o + 127) / 128 * 128;
    sa.stage_bytes = (int)o;
    sa.slot_off = (int)(2 * o);
    sa.max_nslot = max_vm_nslot;
    smem = 2 * o + 12 * (size_t)max_vm_nslot;
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
                          int res_only, cudaStream_t s, bool after_sweep)
{
    void* f = pick_stream(mode, nt);
    if (!f || grid <= 0) return cudaErrorInvalidValue;
    IterArgs ac = a;
    StreamArgs sc = sa;
    void* args[] = {&ac, &sc, &k, &res_only};
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(nt);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    // directly after another sweep: start as a programmatic dependent of it
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr.val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = after_sweep ? 1 : 0;
    return cudaLaunchKernelExC(&cfg, f, args);
}

}  // namespace pdg
