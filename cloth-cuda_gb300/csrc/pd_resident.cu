// Resident persistent PD kernel: one cooperative launch per frame, one patch
// per block for the whole frame.  Each thread keeps its triangle and hinge
// records in registers and its owned vertex's previous offset d^(k-1) in a
// register; the patch's gather lists, y and d^k live in shared memory.  Per
// sweep only the owned offsets go out to L2 and the halo offsets come back.
//
// Synchronisation between sweeps: with fixed sweep counts a block waits only
// for the patches that own its halo vertices (per-patch completion marks in
// global memory); with a residual tolerance every sweep ends in a grid
// barrier, because the convergence decision needs the complete per-cloth
// residual.  Every wait is bounded by a clock64 budget; on expiry the block
// records an error code and leaves, and so do all others at their next wait.
//
// Used when every patch fits one block (nown <= NT, ntri <= MT*NT,
// nhinge <= MH*NT) and all patches are co-resident.
#include "pd_kernels.cuh"
#include "pdg_kernels.h"

namespace pdg {

__device__ __forceinline__ bool grid_barrier_r(unsigned* bar, int* err, long long budget)
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
                if (clock64() - t0 > budget || *(volatile int*)err != 0) { atomicCAS(err, 0, 2); break; }
                __nanosleep(32);
            }
        }
        __threadfence();
        ok = (*(volatile int*)err == 0);
    }
    __syncthreads();
    return ok != 0;
}

__device__ __forceinline__ void st_release_gpu(unsigned long long* p, unsigned long long v)
{
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ unsigned long long ld_acquire_gpu(const unsigned long long* p)
{
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Publish "this patch finished the sweep with mark m" after all of the
// block's global writes (the barrier orders them before thread 0's release).
__device__ __forceinline__ void publish_mark(unsigned long long* pflag, unsigned long long m)
{
    __syncthreads();
    if (threadIdx.x == 0) st_release_gpu(&pflag[blockIdx.x], m);
}

// Wait until every neighbouring patch published a mark >= m (first warp, one
// lane per neighbour, acquire loads), bounded.  Returns false on timeout or a
// prior error.
__device__ __forceinline__ bool wait_neighbours(const int* nb, int nnb, const unsigned long long* pflag,
                                                unsigned long long m, int* err, long long budget)
{
    __shared__ int ok;
    if (threadIdx.x < 32) {
        bool good = true;
        for (int j = threadIdx.x; j < nnb && good; j += 32) {
            const unsigned long long* f = pflag + nb[j];
            const long long t0 = clock64();
            while (ld_acquire_gpu(f) < m) {
                if (clock64() - t0 > budget || *(volatile int*)err != 0) { atomicCAS(err, 0, 3); good = false; break; }
                __nanosleep(20);
            }
        }
        const unsigned all = __ballot_sync(0xffffffffu, good);
        if (threadIdx.x == 0) ok = (all == 0xffffffffu);
    }
    __syncthreads();
    return ok != 0;
}

template <int NT, int MT>
__device__ __forceinline__ int tri_index(int tid, int j)
{
    return j < MT - 1 ? tid + j * NT : (MT - 1) * NT + (NT - 1 - tid);
}

constexpr int kResOmega = 1024;   // Chebyshev weights kept in shared memory

// Local step over this thread's records with list index in [t0, t1) (triangles)
// and [e0, e1) (hinges).
template <int MODE, int NT, int MT, int MH>
__device__ __forceinline__ void local_records(const TriRec (&rt)[MT], const HingeRec (&rh)[MH], const float4* sy,
                                              const float4* sd, int ntri, int nhin, int t0, int t1, int e0, int e1,
                                              float* cx, float* cy, float* cz)
{
    const int tid = threadIdx.x;
    #pragma unroll
    for (int j = 0; j < MT; ++j) {
        const int t = tri_index<NT, MT>(tid, j);
        if (t >= t0 && t < t1) triangle_contrib<MODE>(rt[j], sy, sd, t, ntri, cx, cy, cz);
    }
    #pragma unroll
    for (int j = 0; j < MH; ++j) {
        const int e = tid + j * NT;
        if (e >= e0 && e < e1) hinge_contrib<MODE>(rh[j], sy, sd, e, 3 * ntri, nhin, cx, cy, cz);
    }
}

// Gather and Jacobi update of owned vertex l: o = d^(k+1), d = d^k.
template <int MODE>
__device__ __forceinline__ void vertex_update(const uint16_t* sent, const int* sptr, int l, const float4* sy,
                                              const float4* sd, const float* cx, const float* cy, const float* cz,
                                              float4 dprev, float gamma, float omega, float4& o, float4& d, float& r2)
{
    const float3 f = gather_slots(sent, sptr[l], sptr[l + 1], cx, cy, cz);
    d = sd[l];
    const float4 y = sy[l];
    if (MODE == kModeConsistent) o = update_consistent(d, y, f, dprev, gamma, omega, r2);
    else                         o = update_literal(d, y, f);
}

template <int MODE, int NT, int MT, int MH>
__global__ void __launch_bounds__(NT, 512 / NT) k_resident(PersistArgs p)
{
    extern __shared__ float4 smem[];
    __shared__ PatchHdr ph;
    __shared__ float red[NT / 32];
    __shared__ int skip;
    __shared__ float som[kResOmega];   // Chebyshev weights of this cloth
    const IterArgs& a = p.it;
    const int tid = threadIdx.x;
    if (tid == 0) ph = a.patches[blockIdx.x];
    __syncthreads();
    const int nown = ph.nown, nlocal = ph.nlocal, ntri = ph.ntri, nhin = ph.nhinge;
    float4* sy = smem;
    float4* sd = sy + nlocal;
    float* cx = reinterpret_cast<float*>(sd + nlocal);
    float* cy = cx + ph.nslot;
    float* cz = cy + ph.nslot;
    int* sptr = reinterpret_cast<int*>(cz + ph.nslot);
    uint16_t* sent = reinterpret_cast<uint16_t*>(sptr + nown + 1);

    // records in registers for the whole frame.  The partial last round of
    // triangles goes to the highest threads and that of hinges to the
    // lowest, so warps finish the local step together.
    TriRec rt[MT];
    HingeRec rh[MH];
    #pragma unroll
    for (int j = 0; j < MT; ++j) {
        const int t = tri_index<NT, MT>(tid, j);
        if (t < ntri) rt[j] = a.tris[ph.tri_off + t];
    }
    #pragma unroll
    for (int j = 0; j < MH; ++j) {
        const int e = tid + j * NT;
        if (e < nhin) rh[j] = a.hinges[ph.hinge_off + e];
    }
    // gather lists and Chebyshev weights in shared memory
    for (int l = tid; l <= nown; l += NT) sptr[l] = a.csr_ptr[ph.csr_off + l];
    for (int k = tid; k < a.omega_stride && k < kResOmega; k += NT) som[k] = a.omega[ph.cloth * a.omega_stride + k];
    __syncthreads();
    const int nent = sptr[nown];
    for (int q = tid; q < nent; q += NT) sent[q] = a.csr_ent[ph.ent_off + q];

    // predict the owned vertices; the cloth's first block resets its record
    const int c = ph.cloth;
    const ClothInfo& ci = a.cinfo[c];
    const bool own = tid < nown;
    const bool first = (int)blockIdx.x == ci.patch_begin;
    const int g = ph.vbegin + tid;
    float4 dprev = make_float4(0.f, 0.f, 0.f, 0.f);
    if (first) reset_rt(a.crt, a.acc, a.acc_stride, c, tid, NT);
    if (own) {
        predict_vertex(g, p.X, p.V, p.aux, p.mass, p.vcloth, a.cinfo, p.warm, p.Y, a.buf[0], a.buf[1]);
        dprev = __ldcg(&a.buf[0][g]);
    }
    if (!grid_barrier_r(p.bar, p.err, p.spin_budget)) return;
    for (int l = tid; l < nlocal; l += NT) {
        const int gg = l < nown ? ph.vbegin + l : __ldg(&a.halo[ph.halo_off + l - nown]);
        sy[l] = __ldcg(&a.Y[gg]);
        sd[l] = __ldcg(&a.buf[0][gg]);
    }
    // this thread's first halo vertex, re-read every sweep
    const int hl0 = nown + tid;
    const int hg0 = hl0 < nlocal ? __ldg(&a.halo[ph.halo_off + tid]) : 0;

    const float gamma = ci.gamma;
    const int nsweep = p.max_iter + (p.have_final ? 1 : 0);
    const bool nbr = p.nbr_sync != 0;
    const unsigned long long mark0 = p.frame_seq * (unsigned long long)(nsweep + 2);
    const int* nb = p.nbr + p.nbr_ptr[blockIdx.x];
    const int nnb = p.nbr_ptr[blockIdx.x + 1] - p.nbr_ptr[blockIdx.x];
    double* acc = a.acc + (size_t)c * a.acc_stride;
    for (int k = 0; k < nsweep; ++k) {
        // With fixed sweep counts the cap alone decides (the record stays
        // active through the sweeps), so no thread waits on global memory
        // for it; a tolerance needs the per-cloth decision.
        if (!nbr && tid == 0) skip = cloth_done(a, c, k, first, true) ? 1 : 0;
        if (k > 0) {   // halo offsets d^k written by the neighbouring blocks
            if (nbr && !wait_neighbours(nb, nnb, p.pflag, mark0 + k, p.err, p.spin_budget)) return;
            const float4* Dk = (k & 1) ? a.buf[1] : a.buf[0];
            if (hl0 < nlocal) sd[hl0] = __ldcg(&Dk[hg0]);
            for (int l = hl0 + NT; l < nlocal; l += NT) sd[l] = __ldcg(&Dk[__ldg(&a.halo[ph.halo_off + l - nown])]);
        }
        __syncthreads();
        const bool skip_k = nbr ? (k >= ci.max_iter && (k > ci.max_iter || !a.have_final)) : skip != 0;
        const float omega_k = k < a.omega_stride ? (k < kResOmega ? som[k] : a.omega[c * a.omega_stride + k]) : 1.f;
        const bool res_only = k >= ci.max_iter;
        // Phase A: the records through boundary vertices (a prefix of each
        // list), then the update of the boundary vertices, which the
        // neighbouring patches read: they are published before phase B, so
        // the exchange overlaps the interior's work.
        float4 o = make_float4(0.f, 0.f, 0.f, 0.f), d = o;
        float r2 = 0.f;
        if (!skip_k) {
            local_records<MODE, NT, MT, MH>(rt, rh, sy, sd, ntri, nhin, 0, ph.ntri_a, 0, ph.nhin_a, cx, cy, cz);
            __syncthreads();
            if (tid < ph.nbnd) {
                vertex_update<MODE>(sent, sptr, tid, sy, sd, cx, cy, cz, dprev, gamma, omega_k, o, d, r2);
                if (!res_only) ((k & 1) ? a.buf[0] : a.buf[1])[g] = o;
            }
        }
        if (nbr) publish_mark(p.pflag, mark0 + k + 1);
        if (!skip_k) {
            // Phase B: the remaining records, then the interior vertices
            local_records<MODE, NT, MT, MH>(rt, rh, sy, sd, ntri, nhin, ph.ntri_a, ntri, ph.nhin_a, nhin, cx, cy,
                                            cz);
            __syncthreads();
            if (own && tid >= ph.nbnd) {
                vertex_update<MODE>(sent, sptr, tid, sy, sd, cx, cy, cz, dprev, gamma, omega_k, o, d, r2);
                if (!res_only) ((k & 1) ? a.buf[0] : a.buf[1])[g] = o;
            }
            // every record has read d^k: the owned offsets move on
            if (own && !res_only) {
                sd[tid] = o;
                dprev = d;
            }
            // fixed sweep counts read only the residual of the start and of
            // the last sweeps; a tolerance needs every sweep's
            if (MODE == kModeConsistent && (!nbr || k == 0 || k >= ci.max_iter - 1))
                block_residual<NT>(r2, red, acc + k);
        }
        if (!nbr && !grid_barrier_r(p.bar, p.err, p.spin_budget)) return;
    }
    // every per-sweep sum is complete after this barrier
    if (nbr && !grid_barrier_r(p.bar, p.err, p.spin_budget)) return;
    if (first && tid == 0) frame_stats_cloth(a, c);
    if (!grid_barrier_r(p.bar, p.err, p.spin_budget)) return;
    if (own) finalize_vertex(g, p.Xw, p.V, p.Y, a.buf[0], a.buf[1], p.aux, p.vcloth, a.cinfo, a.crt);
}

// MT x NT triangles and MH x NT hinges per block.  512 threads: one block
// (one patch) per SM; 256 threads: two half-size patches per SM, so one
// block computes while the other waits for its neighbours.  The smaller
// record set (fewer registers) is used when the patches fit it.
struct ResVariant { int nt, mt, mh; void* f[2]; };

static const ResVariant* res_variants(int* n)
{
    static const ResVariant v[] = {
        {512, 2, 3, {(void*)k_resident<kModeConsistent, 512, 2, 3>, (void*)k_resident<kModeLiteral, 512, 2, 3>}},
        {512, 3, 4, {(void*)k_resident<kModeConsistent, 512, 3, 4>, (void*)k_resident<kModeLiteral, 512, 3, 4>}},
        {256, 3, 4, {(void*)k_resident<kModeConsistent, 256, 3, 4>, (void*)k_resident<kModeLiteral, 256, 3, 4>}},
    };
    *n = 3;
    return v;
}

int resident_pick(int nt, int max_ntri, int max_nhinge)
{
    int n = 0;
    const ResVariant* v = res_variants(&n);
    for (int i = 0; i < n; ++i)
        if (v[i].nt == nt && max_ntri <= v[i].mt * nt && max_nhinge <= v[i].mh * nt) return i;
    return -1;
}

static void* variant_fn(int variant, int mode)
{
    int n = 0;
    const ResVariant* v = res_variants(&n);
    if (variant < 0 || variant >= n) return nullptr;
    return v[variant].f[mode == kModeConsistent ? 0 : 1];
}

int resident_max_blocks(int mode, int variant, size_t smem)
{
    void* f = variant_fn(variant, mode);
    if (!f) return 0;
    int n = 0;
    const int nt = res_variants(&n)[variant].nt;
    if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024) != cudaSuccess) return 0;
    int dev = 0, nsm = 0, nb = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, f, nt, smem) != cudaSuccess) return 0;
    return nb * nsm;
}

cudaError_t launch_resident(const PersistArgs& p, int variant, int grid, size_t smem, cudaStream_t s)
{
    void* f = variant_fn(variant, p.mode);
    if (!f || grid <= 0) return cudaErrorInvalidValue;
    int n = 0;
    const int nt = res_variants(&n)[variant].nt;
    PersistArgs copy = p;
    void* args[] = {&copy};
    return cudaLaunchCooperativeKernel(f, dim3(grid), dim3(nt), args, smem, s);
}

}  // namespace pdg
