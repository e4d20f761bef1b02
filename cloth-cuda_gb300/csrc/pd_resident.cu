// Resident persistent PD kernel: one cooperative launch per frame, one patch
// per block for the whole frame.  The patch's cell and hinge records, the
// hinges' slot addresses, the gather pointers, y and d^k live in shared
// memory (vertex-major contribution slots, as in the per-sweep kernels), and
// each thread keeps its owned vertex's previous offset d^(k-1) in a register.  Per sweep only the owned
// offsets go out to L2 and the halo offsets come back.
//
// Synchronisation between sweeps: with fixed sweep counts a block waits only
// for the halo offsets it reads.  Each boundary vertex publishes d^(k+1) as
// three 64-bit words, value bits | tag << 32, with the tag naming the frame
// and the sweep; a reader polls the words of its halo vertices until all
// three carry the tag it expects, so the data itself is the completion flag
// (one write and one read per exchange, no separate mark and no fence).
// With a residual tolerance every sweep ends in a grid barrier, because the
// convergence decision needs the complete per-cloth residual.  Every wait is
// bounded by a clock64 budget; on expiry the block records an error code and
// leaves, and so do all others at their next wait.
//
// Used when every patch fits one block (nown <= NT) and all patches are
// co-resident.
//
// The instance with IO = true also moves the caller's state for the
// host-buffer frame (pdg_solver_step_host): it reads x and v from the caller's
// arrays for the prediction and writes them back after the finalisation, both
// walked in caller order so that page-locked host memory is accessed
// contiguously, which replaces the two copy launches around the frame.
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

// Caller vertex o of an AoS xyz array, or zeros without one.
__device__ __forceinline__ float3 caller_vec(const float* a, int o)
{
    return a ? make_float3(a[3 * o], a[3 * o + 1], a[3 * o + 2]) : make_float3(0.f, 0.f, 0.f);
}

// Predicts layout vertex g from the caller's x and v (xi, vi: its entries in
// the caller's arrays), which replace the solver's state as the scatter copy
// before a frame would have.
__device__ __forceinline__ void predict_caller_vertex(const PersistArgs& p, int g, float3 xi, float3 vi)
{
    const float4 x = p.in_x ? make_float4(xi.x, xi.y, xi.z, 0.f) : __ldcg(&p.X[g]);
    const float4 v = p.in_v ? make_float4(vi.x, vi.y, vi.z, 0.f) : __ldcg(&p.V[g]);
    if (p.in_x) p.Xw[g] = x;
    if (p.in_v) p.V[g] = v;
    predict_vertex_xv(g, x, v, p.aux, p.mass, p.vcloth, p.it.cinfo, p.warm, p.Y, p.it.buf[0], p.it.buf[1]);
}

// Layout vertex g's state into the caller's arrays at caller vertex o (the
// gather copy after a frame).
__device__ __forceinline__ void store_frame_state(const PersistArgs& p, int o, int g)
{
    if (p.out_x) {
        const float4 x = __ldcg(&p.Xw[g]);
        p.out_x[3 * o] = x.x; p.out_x[3 * o + 1] = x.y; p.out_x[3 * o + 2] = x.z;
    }
    if (p.out_v) {
        const float4 v = __ldcg(&p.V[g]);
        p.out_v[3 * o] = v.x; p.out_v[3 * o + 1] = v.y; p.out_v[3 * o + 2] = v.z;
    }
}

// Named barriers (barrier 0 is __syncthreads).  `count` threads, a multiple
// of 32, take part.
__device__ __forceinline__ void named_sync(int id, int count)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

// named_sync that also returns whether `v` held on every taking part thread.
__device__ __forceinline__ bool named_and(int id, int count, bool v)
{
    unsigned r;
    asm volatile("{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\t"
                 "barrier.red.and.pred q, %2, %3, p;\n\tselp.u32 %0, 1, 0, q;\n\t}"
                 : "=r"(r)
                 : "r"((unsigned)v), "r"(id), "r"(count)
                 : "memory");
    return r != 0;
}

// Tagged exchange of one vertex offset: each component is one 64-bit word
// (value bits | tag << 32).  A 64-bit access is single-copy atomic, so a
// reader that finds `tag` in all three words holds the value written with
// it; the words are read and written at GPU scope, bypassing L1.
__device__ __forceinline__ void st_tagged(unsigned long long* w, float4 o, unsigned tag)
{
    const unsigned long long t = (unsigned long long)tag << 32;
    const unsigned long long a = t | __float_as_uint(o.x), b = t | __float_as_uint(o.y), c = t | __float_as_uint(o.z);
    asm volatile("st.relaxed.gpu.global.v2.u64 [%0], {%1, %2};" ::"l"(w), "l"(a), "l"(b) : "memory");
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(w + 2), "l"(c) : "memory");
}

// Reads the words of one vertex; true (and v.xyz set) when all carry `tag`.
__device__ __forceinline__ bool ld_tagged(const unsigned long long* w, unsigned tag, float4& v)
{
    unsigned long long a, b, c;
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(a), "=l"(b) : "l"(w) : "memory");
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(c) : "l"(w + 2) : "memory");
    if ((unsigned)(a >> 32) != tag || (unsigned)(b >> 32) != tag || (unsigned)(c >> 32) != tag) return false;
    v.x = __uint_as_float((unsigned)a);
    v.y = __uint_as_float((unsigned)b);
    v.z = __uint_as_float((unsigned)c);
    return true;
}

// The three words of one vertex, read once (no tag check).
__device__ __forceinline__ void ld_words(const unsigned long long* w, unsigned long long& a, unsigned long long& b,
                                         unsigned long long& c)
{
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(a), "=l"(b) : "l"(w) : "memory");
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(c) : "l"(w + 2) : "memory");
}

// Polls one vertex's words until they carry `tag`, bounded by the clock64
// budget; false on timeout or when another block reported an error.
__device__ __forceinline__ bool poll_tagged(const unsigned long long* w, unsigned tag, float4& v, int* err,
                                            long long budget)
{
    if (ld_tagged(w, tag, v)) return true;
    const long long t0 = clock64();
    for (;;) {
        if (ld_tagged(w, tag, v)) return true;
        if (clock64() - t0 > budget || *(volatile int*)err != 0) {
            atomicCAS(err, 0, 3);
            return false;
        }
    }
}

constexpr int kResOmega = 1024;   // Chebyshev weights kept in shared memory

// Local step over the records with list index in [t0, t1) (cells) and
// [e0, e1) (lone hinges), read from the patch's copy in shared memory.  With
// `rev` the records go to the threads in reverse order (the last thread takes
// the first record), which leaves the first threads free; a record's
// contributions and slots do not depend on the thread that computes them.
template <int MODE, int NT>
__device__ __forceinline__ void local_records(const CellRec* rc, const HingeRec* rh, const uint2* hvs,
                                              const float4* sy, const float4* sd, int ncell, int nhin, int t0, int t1,
                                              int e0, int e1, float2* cxy, float* cz, bool rev = false)
{
    const int j0 = rev ? NT - 1 - (int)threadIdx.x : (int)threadIdx.x;
    for (int t = t0 + j0; t < t1; t += NT) cell_contrib_vm_p<MODE>(rc[t], sy, sd, cxy, cz);
    for (int e = e0 + j0; e < e1; e += NT) hinge_contrib_vm<MODE>(rh[e], hvs[e], sy, sd, cxy, cz);
}

// Jacobi update of owned vertex l with force f: o = d^(k+1), d = d^k.
template <int MODE>
__device__ __forceinline__ void vertex_update_f(float3 f, int l, const float4* sy, const float4* sd, float4 dprev,
                                                float gamma, float omega, float4& o, float4& d, float& r2)
{
    d = sd[l];
    const float4 y = sy[l];
    if (MODE == kModeConsistent) o = update_consistent(d, y, f, dprev, gamma, omega, r2);
    else                         o = update_literal(d, y, f);
}

// Gather by one thread and update.
template <int MODE>
__device__ __forceinline__ void vertex_update(int npad, const int* sptr, int l, const float4* sy,
                                              const float4* sd, const float2* cxy, const float* cz,
                                              float4 dprev, float gamma, float omega, float4& o, float4& d, float& r2)
{
    const int deg = sptr[l + 1] - sptr[l], h = gather_half(deg);
    const float3 f = deg <= 10 ? fadd3(gather_vm_u<5>(l, 0, h, npad, cxy, cz), gather_vm_u<5>(l, h, deg, npad, cxy, cz))
                               : fadd3(gather_vm(l, 0, h, npad, cxy, cz), gather_vm(l, h, deg, npad, cxy, cz));
    vertex_update_f<MODE>(f, l, sy, sd, dprev, gamma, omega, o, d, r2);
}

// Block sum of r2 over the NT compute threads (named barrier 1), added to
// *acc by one double atomic.
template <int NT>
__device__ __forceinline__ void compute_residual(float r2, float* red, double* acc)
{
    const int tid = threadIdx.x;
    r2 = warp_sum(r2);
    if ((tid & 31) == 0) red[tid >> 5] = r2;
    named_sync(1, NT);
    if (tid < 32) {
        float v = tid < NT / 32 ? red[tid] : 0.f;
        v = warp_sum(v);
        if (tid == 0) atomicAdd(acc, (double)v);
    }
}

// Block layout: NT compute threads (thread l < nown owns local vertex l;
// the patch's records in shared memory) and 32 more threads that help stage
// the records at the start of the frame and otherwise only take part in the
// block-wide barriers.  (They were the signal warp of a completion-mark
// protocol, which the tagged exchange replaced: 257x257 sweep 5.5 -> 4.7 us,
// 33x33 4.8 -> 4.3 us, bitwise equal.)
//
// Fixed sweep counts (neighbour synchronisation), one sweep of the compute
// threads:
//   [k > 0: poll the halo's tagged d^k words into shared memory] -> bar 1
//   (a vote: a failed poll makes every compute thread leave the sweep loop)
//   -> phase A records -> bar 1 -> update of the boundary vertices (d^(k+1)
//   to global memory and as tagged words) -> phase B records -> bar 1 ->
//   [first read of the next sweep's halo words] -> interior update.
// Barrier 1 counts the NT compute threads.  With a tolerance every sweep ends
// in a grid barrier instead.
// IO: the instance that also moves the caller's state (p.in_x ... p.out_v);
// the other one compiles without that code.
template <int MODE, int NT, bool IO>
__global__ void __launch_bounds__(NT + 32, 512 / (NT + 32)) k_resident(PersistArgs p)
{
    constexpr int NTT = NT + 32;   // a multiple of 128: 4 warps per SM sub-partition
    extern __shared__ float4 smem[];
    __shared__ PatchHdr ph;
    __shared__ float red[NTT / 32];
    __shared__ int skip;
    __shared__ float som[kResOmega];   // Chebyshev weights of this cloth
    const IterArgs& a = p.it;
    const int tid = threadIdx.x;
    const bool comp = tid < NT;
    // With caller arrays, this thread's first caller vertex is loaded before
    // the patch's records are staged: the host round trip overlaps the staging.
    const bool caller_in = IO && (p.in_x || p.in_v), caller_out = IO && (p.out_x || p.out_v);
    const int o0 = (int)blockIdx.x * NT + tid;
    float3 xi0 = make_float3(0.f, 0.f, 0.f), vi0 = xi0;
    int gi0 = 0;
    if (caller_in && comp && o0 < p.n) {
        gi0 = __ldg(&p.io_inv[o0]);
        xi0 = caller_vec(p.in_x, o0);
        vi0 = caller_vec(p.in_v, o0);
    }
    if (tid == 0) ph = a.patches[blockIdx.x];
    __syncthreads();
    const int nown = ph.nown, nlocal = ph.nlocal, ncell = ph.ncell, nhin = ph.nhinge;
    // shared memory: the patch's records (read every sweep), the hinges' slot
    // addresses, y and d of the local vertices, the vertex-major contribution
    // slots and the gather pointers
    CellRec* rc = reinterpret_cast<CellRec*>(smem);
    HingeRec* rh = reinterpret_cast<HingeRec*>(rc + ncell);
    uint2* hvs = reinterpret_cast<uint2*>(rh + nhin);
    float4* sy = reinterpret_cast<float4*>(hvs + ((nhin + 1) & ~1));
    float4* sd = sy + nlocal;
    float2* cxy = reinterpret_cast<float2*>(sd + nlocal);
    float* cz = reinterpret_cast<float*>(cxy + ph.vm_nslot);
    int* sptr = reinterpret_cast<int*>(cz + ph.vm_nslot);
    const int npad = ph.vm_npad;

    {
        // records from the device format (groups of kCellGroup, piece-major),
        // read in that order, into shared memory record after record
        const uint4* src = reinterpret_cast<const uint4*>(a.cells + ph.cell_off);
        uint4* dst = reinterpret_cast<uint4*>(rc);
        const int n4 = (ncell + kCellGroup - 1) / kCellGroup * (9 * kCellGroup);
        for (int q = tid; q < n4; q += NTT) {
            const int grp = q / (9 * kCellGroup), r = q - grp * (9 * kCellGroup);
            const int i = r / kCellGroup, cc = grp * kCellGroup + r % kCellGroup;
            if (cc < ncell) dst[cc * 9 + i] = __ldg(&src[q]);
        }
        const uint4* hsrc = reinterpret_cast<const uint4*>(a.hinges + ph.hinge_off);
        uint4* hdst = reinterpret_cast<uint4*>(rh);
        for (int q = tid; q < 2 * nhin; q += NTT) hdst[q] = __ldg(&hsrc[q]);
        for (int q = tid; q < nhin; q += NTT) hvs[q] = __ldg(&a.hvm[ph.hinge_off + q]);
    }
    // gather pointers (per-vertex contribution counts) and Chebyshev weights
    for (int l = tid; l <= nown; l += NTT) sptr[l] = a.csr_ptr[ph.csr_off + l];
    for (int k = tid; k < a.omega_stride && k < kResOmega; k += NTT) som[k] = a.omega[ph.cloth * a.omega_stride + k];
    __syncthreads();


    // predict the owned vertices, or with caller arrays the vertices in caller
    // order (a grid-stride walk over the compute threads); the cloth's first
    // block resets its record
    const int c = ph.cloth;
    const ClothInfo& ci = a.cinfo[c];
    const bool own = tid < nown;
    const bool first = (int)blockIdx.x == ci.patch_begin;
    const int g = ph.vbegin + tid;
    float4 dprev = make_float4(0.f, 0.f, 0.f, 0.f);
    if (first) reset_rt(a.crt, a.acc, a.acc_stride, c, tid, NTT);
    if (caller_in) {
        if (comp && o0 < p.n) predict_caller_vertex(p, gi0, xi0, vi0);
        for (int o = o0 + (int)gridDim.x * NT; comp && o < p.n; o += (int)gridDim.x * NT)
            predict_caller_vertex(p, __ldg(&p.io_inv[o]), caller_vec(p.in_x, o), caller_vec(p.in_v, o));
    } else if (own) {
        predict_vertex(g, p.X, p.V, p.aux, p.mass, p.vcloth, a.cinfo, p.warm, p.Y, a.buf[0], a.buf[1]);
        dprev = __ldcg(&a.buf[0][g]);
    }
    // The frame's exchange tags: tag0 + k for d^k, tag0 from the device word
    // that the previous frame advanced (so a replayed launch gets new tags).
    // Before the 32-bit tags would wrap, every block clears its boundary
    // vertices' words in both buffers and the frame starts again from 0; the
    // grid barrier below orders the clearing before any neighbour's poll.
    const int nsweep = p.max_iter + (p.have_final ? 1 : 0);
    unsigned tag0 = 0;
    if (p.xch_tag) {
        const unsigned t = __ldcg(p.xch_tag);
        if ((unsigned long long)t + (unsigned long long)nsweep <= 0xffffffffULL) {
            tag0 = t;
        } else {
            for (int q = tid; q < 8 * ph.nbnd; q += NTT) {
                const int l = q >> 3, b = (q >> 2) & 1, w = q & 3;
                p.xch[((size_t)b * (size_t)p.n + (size_t)(ph.vbegin + l)) * 4 + w] = 0ull;
            }
        }
    }
    if (!grid_barrier_r(p.bar, p.err, p.spin_budget)) return;
    // every block has read the word: the next frame's base
    if (p.xch_tag && blockIdx.x == 0 && tid == 0) *p.xch_tag = tag0 + (unsigned)nsweep;
    if (caller_in && own) dprev = __ldcg(&a.buf[0][g]);
    for (int l = tid; l < nlocal; l += NTT) {
        const int gg = l < nown ? ph.vbegin + l : __ldg(&a.halo[ph.halo_off + l - nown]);
        sy[l] = __ldcg(&a.Y[gg]);
        sd[l] = __ldcg(&a.buf[0][gg]);
    }
    // this compute thread's first halo vertex, re-read every sweep
    const int hl0 = nown + tid;
    const int hg0 = (comp && hl0 < nlocal) ? __ldg(&a.halo[ph.halo_off + tid]) : 0;
    __syncthreads();

    const float gamma = ci.gamma;
    const bool nbr = p.nbr_sync != 0;
    double* acc = a.acc + (size_t)c * a.acc_stride;
    if (nbr && comp) {
        // ---- compute threads, neighbour synchronisation ----
        // the words of this thread's first halo vertex for the next sweep, read
        // ahead while the interior is updated: when they already carry the
        // tag the top of the next sweep needs no round trip (257x257 sweep
        // 4.72 -> 4.60 us; read before phase B instead: 4.76 us)
        unsigned long long pw0 = 0, pw1 = 0, pw2 = 0;
        for (int k = 0; k < nsweep; ++k) {
            if (k > 0 && k <= ci.max_iter) {
                // the neighbours' d^k (written in their sweep k - 1, which
                // every sweep up to the cloth's cap has): poll the tagged
                // words of this thread's halo vertices
                const unsigned tag = tag0 + (unsigned)k;
                const unsigned long long* xb = p.xch + (size_t)(k & 1) * (size_t)p.n * 4;
                bool ok = true;
                for (int l = hl0; ok && l < nlocal; l += NT) {
                    const int gg = l == hl0 ? hg0 : __ldg(&a.halo[ph.halo_off + l - nown]);
                    float4 v = sd[l];
                    if (l == hl0 && (unsigned)(pw0 >> 32) == tag && (unsigned)(pw1 >> 32) == tag &&
                        (unsigned)(pw2 >> 32) == tag) {
                        v.x = __uint_as_float((unsigned)pw0);
                        v.y = __uint_as_float((unsigned)pw1);
                        v.z = __uint_as_float((unsigned)pw2);
                    } else {
                        ok = poll_tagged(xb + (size_t)gg * 4, tag, v, p.err, p.spin_budget);
                    }
                    sd[l] = v;
                }
                if (!named_and(1, NT, ok)) break;   // the grid barrier below reports the error
            } else {
                named_sync(1, NT);
            }
            // the cap alone decides: the cloth's record stays active through the sweeps
            const bool skip_k = k >= ci.max_iter && (k > ci.max_iter || !a.have_final);
            const float omega_k =
                k < a.omega_stride ? (k < kResOmega ? som[k] : a.omega[c * a.omega_stride + k]) : 1.f;
            const bool res_only = k >= ci.max_iter;
            float4 o = make_float4(0.f, 0.f, 0.f, 0.f), d = o;
            float r2 = 0.f;
            // Phase A: the records through boundary vertices (a prefix of
            // each list), then the boundary vertices, which the neighbouring
            // patches read: their tagged words go out before phase B runs.
            if (!skip_k)
                local_records<MODE, NT>(rc, rh, hvs, sy, sd, ncell, nhin, 0, ph.ncell_a, 0, ph.nhin_a, cxy, cz);
            named_sync(1, NT);
            // The boundary vertices' sums are on the neighbours' critical path:
            // one thread per vertex, every slot load issued before the
            // additions.  (Splitting each sum over an owner and a helper
            // thread joined by a named barrier, the two halves of its
            // definition, was slower once the loads were hoisted.)
            if (!skip_k && tid < ph.nbnd) {
                vertex_update<MODE>(npad, sptr, tid, sy, sd, cxy, cz, dprev, gamma, omega_k, o, d, r2);
                if (!res_only) {
                    ((k & 1) ? a.buf[0] : a.buf[1])[g] = o;
                    st_tagged(p.xch + ((size_t)((k + 1) & 1) * (size_t)p.n + g) * 4, o, tag0 + (unsigned)(k + 1));
                }
            }
            // Phase B: the remaining records, then the interior vertices.  At
            // most a warp's worth of records goes to the last threads, which
            // are idle while the first ones sum the boundary vertices; a larger
            // phase B stays on the first threads, which reach it after the
            // boundary offsets are out, so that it does not compete with the
            // boundary sums the neighbouring patches wait for.
            if (!skip_k)
                local_records<MODE, NT>(rc, rh, hvs, sy, sd, ncell, nhin, ph.ncell_a, ncell, ph.nhin_a, nhin, cxy,
                                        cz, (ncell - ph.ncell_a) + (nhin - ph.nhin_a) <= 32);
            named_sync(1, NT);
            if (k + 1 < nsweep && k + 1 <= ci.max_iter && hl0 < nlocal)
                ld_words(p.xch + ((size_t)((k + 1) & 1) * (size_t)p.n + hg0) * 4, pw0, pw1, pw2);
            if (!skip_k && own && tid >= ph.nbnd) {
                vertex_update<MODE>(npad, sptr, tid, sy, sd, cxy, cz, dprev, gamma, omega_k, o, d, r2);
                if (!res_only) ((k & 1) ? a.buf[0] : a.buf[1])[g] = o;
            }
            // every record has read d^k: the owned offsets move on
            if (!skip_k && own && !res_only) {
                sd[tid] = o;
                dprev = d;
            }
            // fixed sweep counts read only the residual of the start and of
            // the last sweeps
            if (MODE == kModeConsistent && !skip_k && (k == 0 || k >= ci.max_iter - 1))
                compute_residual<NT>(r2, red, acc + k);
        }
    } else if (!nbr) {
        // ---- tolerance: every sweep ends in a grid barrier ----
        for (int k = 0; k < nsweep; ++k) {
            if (tid == 0) skip = cloth_done(a, c, k, first, true) ? 1 : 0;
            if (k > 0 && comp) {
                const float4* Dk = (k & 1) ? a.buf[1] : a.buf[0];
                if (hl0 < nlocal) sd[hl0] = __ldcg(&Dk[hg0]);
                for (int l = hl0 + NT; l < nlocal; l += NT) sd[l] = __ldcg(&Dk[__ldg(&a.halo[ph.halo_off + l - nown])]);
            }
            __syncthreads();
            const bool skip_k = skip != 0;
            const float omega_k =
                k < a.omega_stride ? (k < kResOmega ? som[k] : a.omega[c * a.omega_stride + k]) : 1.f;
            const bool res_only = k >= ci.max_iter;
            float4 o = make_float4(0.f, 0.f, 0.f, 0.f), d = o;
            float r2 = 0.f;
            if (!skip_k) {
                if (comp) local_records<MODE, NT>(rc, rh, hvs, sy, sd, ncell, nhin, 0, ncell, 0, nhin, cxy, cz);
                __syncthreads();
                if (own) {
                    vertex_update<MODE>(npad, sptr, tid, sy, sd, cxy, cz, dprev, gamma, omega_k, o, d, r2);
                    if (!res_only) {
                        ((k & 1) ? a.buf[0] : a.buf[1])[g] = o;
                        sd[tid] = o;
                        dprev = d;
                    }
                }
                if (MODE == kModeConsistent) block_residual<NTT>(r2, red, acc + k);
            }
            if (!grid_barrier_r(p.bar, p.err, p.spin_budget)) return;
        }
    }
    // every per-sweep sum is complete after this barrier
    if (nbr && !grid_barrier_r(p.bar, p.err, p.spin_budget)) return;
    if (first && tid == 0) frame_stats_cloth(a, c);
    if (!grid_barrier_r(p.bar, p.err, p.spin_budget)) return;
    if (caller_out) {
        for (int o = o0; comp && o < p.n; o += (int)gridDim.x * NT) {
            const int gv = __ldg(&p.io_inv[o]);
            finalize_vertex(gv, p.Xw, p.V, p.Y, a.buf[0], a.buf[1], p.aux, p.vcloth, a.cinfo, a.crt);
            store_frame_state(p, o, gv);
        }
    } else if (own) {
        finalize_vertex(g, p.Xw, p.V, p.Y, a.buf[0], a.buf[1], p.aux, p.vcloth, a.cinfo, a.crt);
    }
}

// NT compute threads plus one warp: 480 + 32 threads, one block (one patch)
// per SM; 224 + 32, two half-size patches per SM.  Instances: the
// consistent solve, the reference-literal solve, and the consistent solve
// that moves the caller's state.
struct ResVariant { int nt; void* f[3]; };

static const ResVariant* res_variants(int* n)
{
    static const ResVariant v[] = {
        {480, {(void*)k_resident<kModeConsistent, 480, false>, (void*)k_resident<kModeLiteral, 480, false>,
               (void*)k_resident<kModeConsistent, 480, true>}},
        {224, {(void*)k_resident<kModeConsistent, 224, false>, (void*)k_resident<kModeLiteral, 224, false>,
               (void*)k_resident<kModeConsistent, 224, true>}},
    };
    *n = 2;
    return v;
}

int resident_pick(int nt)
{
    int n = 0;
    const ResVariant* v = res_variants(&n);
    for (int i = 0; i < n; ++i)
        if (v[i].nt == nt) return i;
    return -1;
}

static void* variant_fn(int variant, int mode, bool io)
{
    int n = 0;
    const ResVariant* v = res_variants(&n);
    if (variant < 0 || variant >= n) return nullptr;
    if (io) return mode == kModeConsistent ? v[variant].f[2] : nullptr;
    return v[variant].f[mode == kModeConsistent ? 0 : 1];
}

bool resident_moves_state(int mode) { return mode == kModeConsistent; }

int resident_max_blocks(int mode, int variant, size_t smem)
{
    void* f = variant_fn(variant, mode, false);
    if (!f) return 0;
    int n = 0;
    const int nt = res_variants(&n)[variant].nt;
    for (void* fi : {f, variant_fn(variant, mode, true)})
        if (fi && cudaFuncSetAttribute(fi, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024) != cudaSuccess)
            return 0;
    int dev = 0, nsm = 0, nb = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, f, nt + 32, smem) != cudaSuccess) return 0;
    return nb * nsm;
}

cudaError_t launch_resident(const PersistArgs& p, int variant, int grid, size_t smem, cudaStream_t s)
{
    const bool io = p.in_x || p.in_v || p.out_x || p.out_v;
    void* f = variant_fn(variant, p.mode, io);
    if (!f || grid <= 0) return cudaErrorInvalidValue;
    int n = 0;
    const int nt = res_variants(&n)[variant].nt;
    PersistArgs copy = p;
    void* args[] = {&copy};
    return cudaLaunchCooperativeKernel(f, dim3(grid), dim3(nt + 32), args, smem, s);
}

}  // namespace pdg
