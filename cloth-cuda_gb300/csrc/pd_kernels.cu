// Kernels of the PD cloth solve (sm_103a).
//
// One frame (src/pd_solver.cu:496-621, re-designed):
//   k_predict     y = x + h v + h^2 a; x^0 and x^-1 set to the start iterate
//   k_iter  x K   one fused local+global sweep per launch: each block stages
//                 its patch's positions in shared memory, projects every
//                 triangle (closed-form polar) and hinge, writes per-corner
//                 contributions to shared slots, then every owned vertex
//                 gathers its slots in a fixed order (no atomics, bitwise
//                 deterministic), forms the Jacobi update with the Chebyshev
//                 blend and adds its residual to a per-cloth sum.
//   k_finalize    v = (x^K - x_n)(1 - damping)/h, x = x^K, pins re-applied
//   k_frame_stats per-cloth bookkeeping of the frame
#include "pd_kernels.cuh"
#include "pdg_kernels.h"

#include <cmath>

namespace pdg {

template <int MODE, int NT>
__global__ void __launch_bounds__(NT, 768 / NT) k_iter(IterArgs a, int k, int res_only)
{
    extern __shared__ float4 smem[];
    __shared__ PatchHdr ph;
    __shared__ float red[NT / 32];
    __shared__ int skip;
    __shared__ float omega;
    if (threadIdx.x == 0) ph = a.patches[blockIdx.x];
    __syncthreads();
    // thread 0 takes the per-cloth decision while the others stage the patch
    if (threadIdx.x == 0) {
        const int c = ph.cloth;
        const ClothInfo& ci = a.cinfo[c];
        skip = cloth_done(a, c, k, (int)blockIdx.x == ci.patch_begin) ? 1 : 0;
        omega = (k < a.omega_stride) ? a.omega[c * a.omega_stride + k] : 1.f;
    }
    float4* sx = smem;
    float2* cxy = reinterpret_cast<float2*>(sx + 2 * ph.nlocal);
    float* cz = reinterpret_cast<float*>(cxy + ph.vm_nslot);
    process_patch<MODE, NT>(a, ph, k, res_only != 0 || k >= a.cinfo[ph.cloth].max_iter, 1.f, sx, cxy, cz, red,
                            &skip, &omega);
}

// Residual of the offsets D (no update) into acc[cloth][slot]: one block per patch.
template <int NT>
__global__ void __launch_bounds__(NT) k_res_eval(IterArgs a, const float4* D, int slot)
{
    extern __shared__ float4 smem[];
    __shared__ PatchHdr ph;
    __shared__ float red[NT / 32];
    if (threadIdx.x == 0) ph = a.patches[blockIdx.x];
    __syncthreads();
    IterArgs b = a;
    b.buf[0] = b.buf[1] = const_cast<float4*>(D);
    b.acc = a.acc + slot;
    float4* sx = smem;
    float2* cxy = reinterpret_cast<float2*>(sx + 2 * ph.nlocal);
    float* cz = reinterpret_cast<float*>(cxy + ph.vm_nslot);
    process_patch<kModeConsistent, NT>(b, ph, 0, true, 1.f, sx, cxy, cz, red);
}

// Keep the learned start of a cloth only if its residual is below the
// inertial start's; record r(y) as the frame's normaliser.
__global__ void k_select_cloth(IterArgs a, int slot_y, int slot_w)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.ncloth) return;
    const double r2y = a.acc[(size_t)c * a.acc_stride + slot_y];
    const double r2w = a.acc[(size_t)c * a.acc_stride + slot_w];
    ClothRT& rt = a.crt[c];
    const int init = a.cinfo[c].init;
    rt.warm = ((init == 2 && r2w < r2y) || init == 3) && isfinite(r2w) ? 1 : 0;
    rt.res_y2 = r2y;
}

__global__ void k_select_vertex(int n, const int* __restrict__ vcloth, const ClothRT* __restrict__ crt,
                                const float4* __restrict__ warm, float4* __restrict__ A, float4* __restrict__ B)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !crt[vcloth[i]].warm) return;
    const float4 w = warm[i];
    A[i] = w;
    B[i] = w;
}

// Learned start judged after K sweeps: the inertial chain (buf, crt, acc)
// and the learned chain (b) run K sweeps each from their own start; then
// every cloth continues from the chain with the lower residual.
// Start of the learned chain: per cloth its record (normaliser r(y)^2 from
// the inertial start's evaluation in acc[slot_y], also given to the
// inertial chain; 0 when slot_y < 0, in which case k_warm_start_norm sets it
// after the inertial chain's first sweep) and cleared per-sweep sums; one
// block per cloth.
__global__ void k_warm_init_cloth(IterArgs a, IterArgs b, int slot_y)
{
    const int c = blockIdx.x;
    const double r2y = slot_y >= 0 ? a.acc[(size_t)c * a.acc_stride + slot_y] : 0.0;
    if (threadIdx.x == 0) {
        a.crt[c].res_y2 = r2y;
        if (a.cinfo[c].init == 3) a.crt[c].warm = 1;
        ClothRT r;
        r.active = 1; r.used = 0; r.status = 0; r.warm = 1;
        r.res_y2 = r2y; r.res0_2 = 0.0; r.resf_2 = -1.0;
        b.crt[c] = r;
    }
    for (int k = threadIdx.x; k < b.acc_stride; k += blockDim.x) b.acc[(size_t)c * b.acc_stride + k] = 0.0;
}

// The normaliser of both chains from the inertial chain's first sweep: that
// sweep's residual sum acc[0] is r(x^0)^2 of the chain's start offsets, the
// value k_res_eval gives for them (used when no cloth starts the inertial
// chain from the prediction, i.e. none always keeps it).  One thread per
// cloth, between the inertial chain's sweeps 0 and 1.
__global__ void k_warm_start_norm(IterArgs a, IterArgs b)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.ncloth) return;
    const double r2y = __ldcg(&a.acc[(size_t)c * a.acc_stride]);
    a.crt[c].res_y2 = r2y;
    b.crt[c].res_y2 = r2y;
}

// Start iterates of both chains: the learned chain starts from the
// prediction (cloths asking for the judged learned start) or the inertial
// start (others); cloths that always keep the prediction start from it on
// the inertial chain too.
__global__ void k_warm_init_vertex(int n, const int* __restrict__ vcloth, const ClothInfo* __restrict__ cinfo,
                                   const float4* __restrict__ warm, float4* __restrict__ A, float4* __restrict__ B,
                                   float4* __restrict__ A2, float4* __restrict__ B2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int init = cinfo[vcloth[i]].init;
    const float4 s = init >= 2 ? warm[i] : A[i];
    if (init == 3) { A[i] = s; B[i] = s; }
    A2[i] = s;
    B2[i] = s;
}

// The judge after K sweeps, one thread per cloth asking for the judged
// learned start: each chain's last evaluated residual (that of x^(K-1) while
// the chain iterates, its final one if it stopped; +inf after a failure or
// without one) decides, ties to the inertial chain.  The learned chain's
// record and per-sweep sums replace the inertial chain's when it wins.
__global__ void k_judge_cloth(IterArgs a, IterArgs b, int K)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.ncloth || a.cinfo[c].init != 2) return;
    const double inf = __longlong_as_double(0x7ff0000000000000LL);
    auto eff = [&](const ClothRT& r, const double* acc) {
        double v = r.status != 0 ? inf : (r.active ? acc[K - 1] : (r.resf_2 >= 0.0 ? r.resf_2 : inf));
        return isfinite(v) ? v : inf;
    };
    double* am = a.acc + (size_t)c * a.acc_stride;
    const double* al = b.acc + (size_t)c * b.acc_stride;
    const ClothRT rm = a.crt[c], rl = b.crt[c];
    if (!(eff(rl, al) < eff(rm, am))) return;
    ClothRT r = rl;
    r.warm = 1;
    r.res_y2 = rm.res_y2;
    a.crt[c] = r;
    for (int k = 0; k < a.acc_stride - 2; ++k) am[k] = al[k];
}

// Vertices of cloths whose learned chain won take its iterates d^K, d^(K-1).
__global__ void k_judge_vertex(int n, const int* __restrict__ vcloth, const ClothInfo* __restrict__ cinfo,
                               const ClothRT* __restrict__ crt, float4* __restrict__ A, float4* __restrict__ B,
                               const float4* __restrict__ A2, const float4* __restrict__ B2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = vcloth[i];
    if (cinfo[c].init != 2 || !crt[c].warm) return;
    A[i] = A2[i];
    B[i] = B2[i];
}

__global__ void k_predict(const float4* __restrict__ X, const float4* __restrict__ V,
                          const float4* __restrict__ aux, const float* __restrict__ mass,
                          const int* __restrict__ vcloth, const ClothInfo* __restrict__ cinfo,
                          const float4* __restrict__ warm, float4* __restrict__ Y,
                          float4* __restrict__ A, float4* __restrict__ B, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) predict_vertex(i, X, V, aux, mass, vcloth, cinfo, warm, Y, A, B);
}

// one block per cloth
__global__ void k_reset_rt(ClothRT* crt, double* acc, int acc_stride)
{
    reset_rt(crt, acc, acc_stride, blockIdx.x, threadIdx.x, blockDim.x);
}

__global__ void k_frame_stats(IterArgs a)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < a.ncloth) frame_stats_cloth(a, c);
}

__global__ void k_finalize(float4* __restrict__ X, float4* __restrict__ V, const float4* __restrict__ Y,
                           const float4* __restrict__ A, const float4* __restrict__ B,
                           const float4* __restrict__ aux, const int* __restrict__ vcloth,
                           const ClothInfo* __restrict__ cinfo, const ClothRT* __restrict__ crt, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) finalize_vertex(i, X, V, Y, A, B, aux, vcloth, cinfo, crt);
}

// AoS xyz (caller order, cloth by cloth) <-> float4 reordered.
// Caller-order AoS xyz -> solver-order float4 (w = 0), for one or two
// arrays per launch (x and v of a state copy).
// The state a caller writes replaces the solver's; where it differs from the
// solver's own (bitwise), the vertex's previous-frame offset kept for the
// learned start (dprev, may be null) no longer belongs to its trajectory
// and is marked invalid.
__device__ __forceinline__ bool put_differs(float4 old, float x, float y, float z)
{
    return __float_as_uint(old.x) != __float_as_uint(x) || __float_as_uint(old.y) != __float_as_uint(y) ||
           __float_as_uint(old.z) != __float_as_uint(z);
}

__global__ void k_scatter_state(const float* __restrict__ src0, float4* __restrict__ dst0,
                                const float* __restrict__ src1, float4* __restrict__ dst1,
                                const int* __restrict__ perm_global, int n, float4* __restrict__ dprev)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int o = perm_global[i];
    bool moved = false;
    if (src0) {
        const float4 a = make_float4(src0[3 * o], src0[3 * o + 1], src0[3 * o + 2], 0.f);
        if (dprev) moved = put_differs(dst0[i], a.x, a.y, a.z);
        dst0[i] = a;
    }
    if (src1) {
        const float4 a = make_float4(src1[3 * o], src1[3 * o + 1], src1[3 * o + 2], 0.f);
        if (dprev) moved = moved || put_differs(dst1[i], a.x, a.y, a.z);
        dst1[i] = a;
    }
    if (moved) dprev[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

__global__ void k_gather_state(const float4* __restrict__ src0, float* __restrict__ dst0,
                               const float4* __restrict__ src1, float* __restrict__ dst1,
                               const int* __restrict__ perm_global, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int o = perm_global[i];
    if (dst0) { const float4 v = src0[i]; dst0[3 * o] = v.x; dst0[3 * o + 1] = v.y; dst0[3 * o + 2] = v.z; }
    if (dst1) { const float4 v = src1[i]; dst1[3 * o] = v.x; dst1[3 * o + 1] = v.y; dst1[3 * o + 2] = v.z; }
}

// The same copies walked in caller order through the inverse permutation,
// so the caller-side buffers (page-locked host memory accessed in place)
// are read and written contiguously.
__global__ void k_put_state(const float* __restrict__ x, const float* __restrict__ v, float4* __restrict__ X,
                            float4* __restrict__ V, const int* __restrict__ inv, int n, float4* __restrict__ dprev)
{
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= n) return;
    const int i = inv[o];
    bool moved = false;
    if (x) {
        const float4 a = make_float4(x[3 * o], x[3 * o + 1], x[3 * o + 2], 0.f);
        if (dprev) moved = put_differs(X[i], a.x, a.y, a.z);
        X[i] = a;
    }
    if (v) {
        const float4 a = make_float4(v[3 * o], v[3 * o + 1], v[3 * o + 2], 0.f);
        if (dprev) moved = moved || put_differs(V[i], a.x, a.y, a.z);
        V[i] = a;
    }
    if (moved) dprev[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

__global__ void k_take_state(const float4* __restrict__ X, const float4* __restrict__ V, float* __restrict__ x,
                             float* __restrict__ v, const int* __restrict__ inv, int n)
{
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= n) return;
    const int i = inv[o];
    if (x) { const float4 a = X[i]; x[3 * o] = a.x; x[3 * o + 1] = a.y; x[3 * o + 2] = a.z; }
    if (v) { const float4 a = V[i]; v[3 * o] = a.x; v[3 * o + 1] = a.y; v[3 * o + 2] = a.z; }
}

// apply_constraints_kernel (src/pd_solver.cu:414-428) on AoS device arrays.
__global__ void k_apply_pins(float* __restrict__ pos, float* __restrict__ vel, const int* __restrict__ idx,
                             const float* __restrict__ target, int P)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    const int v = idx[i];
    pos[3 * v] = target[3 * i]; pos[3 * v + 1] = target[3 * i + 1]; pos[3 * v + 2] = target[3 * i + 2];
    if (vel) { vel[3 * v] = 0.f; vel[3 * v + 1] = 0.f; vel[3 * v + 2] = 0.f; }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static inline int nblk(int n, int b) { return (n + b - 1) / b; }

template <int MODE, int NT>
// The shared/L1 split is a property of the kernel function: it is set when
// it differs from the last value set for this instance (carveout 0 = the
// driver's choice).
static cudaError_t launch_iter_t(const IterArgs& a, int npatch, size_t smem, int k, int res_only, int carveout,
                                 cudaStream_t s)
{
    static bool attr_set = false;   // per template instance
    static int carve_set = 0;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(k_iter<MODE, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    if (carveout != carve_set) {
        cudaError_t e = cudaFuncSetAttribute(k_iter<MODE, NT>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                             carveout > 0 ? carveout : (int)cudaSharedmemCarveoutDefault);
        if (e != cudaSuccess) return e;
        carve_set = carveout;
    }
    k_iter<MODE, NT><<<npatch, NT, smem, s>>>(a, k, res_only);
    return cudaGetLastError();
}

cudaError_t launch_iter(const IterArgs& a, int mode, int nt, int npatch, size_t smem, int k, int res_only,
                        cudaStream_t s, int carveout)
{
    if (mode == kModeConsistent) {
        switch (nt) {
            case 128: return launch_iter_t<kModeConsistent, 128>(a, npatch, smem, k, res_only, carveout, s);
            case 256: return launch_iter_t<kModeConsistent, 256>(a, npatch, smem, k, res_only, carveout, s);
            case 512: return launch_iter_t<kModeConsistent, 512>(a, npatch, smem, k, res_only, carveout, s);
        }
    } else {
        switch (nt) {
            case 128: return launch_iter_t<kModeLiteral, 128>(a, npatch, smem, k, res_only, carveout, s);
            case 256: return launch_iter_t<kModeLiteral, 256>(a, npatch, smem, k, res_only, carveout, s);
            case 512: return launch_iter_t<kModeLiteral, 512>(a, npatch, smem, k, res_only, carveout, s);
        }
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_predict(const IterArgs& a, const float4* X, const float4* V, const float4* aux,
                           const float* mass, const int* vcloth, const float4* warm, int n, cudaStream_t s)
{
    k_reset_rt<<<a.ncloth, 64, 0, s>>>(a.crt, a.acc, a.acc_stride);
    k_predict<<<nblk(n, 256), 256, 0, s>>>(X, V, aux, mass, vcloth, a.cinfo, warm, const_cast<float4*>(a.Y),
                                           a.buf[0], a.buf[1], n);
    return cudaGetLastError();
}

cudaError_t launch_finalize(const IterArgs& a, float4* X, float4* V, const float4* aux, const int* vcloth, int n,
                            cudaStream_t s)
{
    k_frame_stats<<<nblk(a.ncloth, 128), 128, 0, s>>>(a);
    k_finalize<<<nblk(n, 256), 256, 0, s>>>(X, V, a.Y, a.buf[0], a.buf[1], aux, vcloth, a.cinfo, a.crt, n);
    return cudaGetLastError();
}

cudaError_t launch_warm_select(const IterArgs& a, int nt, int npatch, size_t smem, const float4* warm,
                               const int* vcloth, int n, cudaStream_t s)
{
    const int slot_y = a.acc_stride - 2, slot_w = a.acc_stride - 1;
    static bool attr_set[3] = {false, false, false};
    const int ti = nt == 128 ? 0 : (nt == 256 ? 1 : 2);
    void* f = nt == 128 ? (void*)k_res_eval<128> : (nt == 256 ? (void*)k_res_eval<256> : (void*)k_res_eval<512>);
    if (!attr_set[ti]) {
        const cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        if (e != cudaSuccess) return e;
        attr_set[ti] = true;
    }
    for (int which = 0; which < 2; ++which) {
        const float4* D = which == 0 ? a.buf[0] : warm;
        const int slot = which == 0 ? slot_y : slot_w;
        if (nt == 128) k_res_eval<128><<<npatch, 128, smem, s>>>(a, D, slot);
        else if (nt == 256) k_res_eval<256><<<npatch, 256, smem, s>>>(a, D, slot);
        else k_res_eval<512><<<npatch, 512, smem, s>>>(a, D, slot);
    }
    k_select_cloth<<<nblk(a.ncloth, 128), 128, 0, s>>>(a, slot_y, slot_w);
    k_select_vertex<<<nblk(n, 256), 256, 0, s>>>(n, vcloth, a.crt, warm, a.buf[0], a.buf[1]);
    return cudaGetLastError();
}

cudaError_t launch_warm_chain_init(const IterArgs& a, const IterArgs& b, int nt, int npatch, size_t smem,
                                   const float4* warm, const int* vcloth, int n, bool eval_start, cudaStream_t s)
{
    const int slot_y = a.acc_stride - 2;
    if (!eval_start) {
        k_warm_init_cloth<<<a.ncloth, 64, 0, s>>>(a, b, -1);
        k_warm_init_vertex<<<nblk(n, 256), 256, 0, s>>>(n, vcloth, a.cinfo, warm, a.buf[0], a.buf[1], b.buf[0],
                                                         b.buf[1]);
        return cudaGetLastError();
    }
    static bool attr_set[3] = {false, false, false};
    const int ti = nt == 128 ? 0 : (nt == 256 ? 1 : 2);
    void* f = nt == 128 ? (void*)k_res_eval<128> : (nt == 256 ? (void*)k_res_eval<256> : (void*)k_res_eval<512>);
    if (!attr_set[ti]) {
        const cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        if (e != cudaSuccess) return e;
        attr_set[ti] = true;
    }
    if (nt == 128) k_res_eval<128><<<npatch, 128, smem, s>>>(a, a.buf[0], slot_y);
    else if (nt == 256) k_res_eval<256><<<npatch, 256, smem, s>>>(a, a.buf[0], slot_y);
    else k_res_eval<512><<<npatch, 512, smem, s>>>(a, a.buf[0], slot_y);
    k_warm_init_cloth<<<a.ncloth, 64, 0, s>>>(a, b, slot_y);
    k_warm_init_vertex<<<nblk(n, 256), 256, 0, s>>>(n, vcloth, a.cinfo, warm, a.buf[0], a.buf[1], b.buf[0], b.buf[1]);
    return cudaGetLastError();
}

cudaError_t launch_warm_start_norm(const IterArgs& a, const IterArgs& b, cudaStream_t s)
{
    k_warm_start_norm<<<nblk(a.ncloth, 128), 128, 0, s>>>(a, b);
    return cudaGetLastError();
}

// After a frame: the offset x_{n+1} - y_n of each vertex, valid (w = 1) for
// free vertices of cloths whose solve succeeded; the learned start's feature
// of the next frame.
__global__ void k_keep_offset(int n, const float4* __restrict__ X, const float4* __restrict__ Y,
                              const float4* __restrict__ aux, const int* __restrict__ vcloth,
                              const ClothRT* __restrict__ crt, float4* __restrict__ Dp)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 x = X[i], y = Y[i];
    const bool ok = aux[i].w >= 0.f && crt[vcloth[i]].status == 0;
    Dp[i] = ok ? make_float4(x.x - y.x, x.y - y.y, x.z - y.z, 1.f) : make_float4(0.f, 0.f, 0.f, 0.f);
}

cudaError_t launch_keep_offset(const IterArgs& a, const float4* X, const float4* aux, const int* vcloth, float4* dprev,
                               int n, cudaStream_t s)
{
    k_keep_offset<<<nblk(n, 256), 256, 0, s>>>(n, X, a.Y, aux, vcloth, a.crt, dprev);
    return cudaGetLastError();
}

cudaError_t launch_warm_judge(const IterArgs& a, const IterArgs& b, int K, const int* vcloth, int n, cudaStream_t s)
{
    k_judge_cloth<<<nblk(a.ncloth, 128), 128, 0, s>>>(a, b, K);
    k_judge_vertex<<<nblk(n, 256), 256, 0, s>>>(n, vcloth, a.cinfo, a.crt, a.buf[0], a.buf[1], b.buf[0], b.buf[1]);
    return cudaGetLastError();
}

cudaError_t launch_scatter_state(const float* src, float4* dst, const int* perm, int n, cudaStream_t s,
                                 const float* src1, float4* dst1, float4* dprev)
{
    if (n == 0 || (!src && !src1)) return cudaSuccess;
    k_scatter_state<<<nblk(n, 256), 256, 0, s>>>(src, dst, src1, dst1, perm, n, dprev);
    return cudaGetLastError();
}

cudaError_t launch_gather_state(const float4* src, float* dst, const int* perm, int n, cudaStream_t s,
                                const float4* src1, float* dst1)
{
    if (n == 0 || (!dst && !dst1)) return cudaSuccess;
    k_gather_state<<<nblk(n, 256), 256, 0, s>>>(src, dst, src1, dst1, perm, n);
    return cudaGetLastError();
}

cudaError_t launch_put_state(const float* x, const float* v, float4* X, float4* V, const int* inv, int n,
                             cudaStream_t s, float4* dprev)
{
    if (n == 0 || (!x && !v)) return cudaSuccess;
    k_put_state<<<nblk(n, 256), 256, 0, s>>>(x, v, X, V, inv, n, dprev);
    return cudaGetLastError();
}

cudaError_t launch_take_state(const float4* X, const float4* V, float* x, float* v, const int* inv, int n,
                              cudaStream_t s)
{
    if (n == 0 || (!x && !v)) return cudaSuccess;
    k_take_state<<<nblk(n, 256), 256, 0, s>>>(X, V, x, v, inv, n);
    return cudaGetLastError();
}

cudaError_t launch_apply_pins(float* pos, float* vel, const int* idx, const float* target, int P, cudaStream_t s)
{
    if (P == 0) return cudaSuccess;
    k_apply_pins<<<nblk(P, 256), 256, 0, s>>>(pos, vel, idx, target, P);
    return cudaGetLastError();
}

}  // namespace pdg
