// Solver lifecycle and per-frame orchestration (PDSolver, src/pd_solver.cu:445-621,
// re-designed): layout upload, CUDA-graph or persistent frame, state I/O.
#include "pdg_solver.h"

#include <algorithm>
#include <cmath>
#include <cstring>

using namespace pdg;

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return set_error(e_ == cudaErrorMemoryAllocation ? PDG_ERR_ALLOC : PDG_ERR_CUDA,  \
                             "%s failed: %s", #call, cudaGetErrorString(e_));                 \
    } while (0)

pdg_solver::~pdg_solver()
{
    if (ws) warm_detach(ws);
    if (graph) cudaGraphExecDestroy(graph);
    if (own_stream && stream) cudaStreamDestroy(stream);
}

namespace {

int check_cfg(const pdg_config& c, int i)
{
    if (c.max_iterations < 0 || c.max_iterations > 100000)
        return set_error(PDG_ERR_ARG, "cloth %d: max_iterations out of range", i);
    if (!(c.dt > 0.f) || !std::isfinite(c.dt)) return set_error(PDG_ERR_ARG, "cloth %d: dt must be > 0", i);
    if (!(c.damping >= 0.f && c.damping <= 1.f)) return set_error(PDG_ERR_ARG, "cloth %d: damping must be in [0, 1]", i);
    if (c.use_chebyshev && !(c.rho >= 0.f && c.rho < 1.f))
        return set_error(PDG_ERR_ARG, "cloth %d: rho must be in [0, 1)", i);
    if (!(c.gamma > 0.f && c.gamma <= 2.f)) return set_error(PDG_ERR_ARG, "cloth %d: gamma must be in (0, 2]", i);
    if (c.cheb_delay < 0) return set_error(PDG_ERR_ARG, "cloth %d: cheb_delay must be >= 0", i);
    if (c.mode != PDG_MODE_CONSISTENT && c.mode != PDG_MODE_REFERENCE_LITERAL)
        return set_error(PDG_ERR_ARG, "cloth %d: unknown mode", i);
    if (c.init < 0 || c.init > 3) return set_error(PDG_ERR_ARG, "cloth %d: unknown init", i);
    if (!std::isfinite(c.gravity) || !std::isfinite(c.wind[0]) || !std::isfinite(c.wind[1]) || !std::isfinite(c.wind[2]))
        return set_error(PDG_ERR_ARG, "cloth %d: non-finite acceleration", i);
    return PDG_OK;
}

int upload_all(pdg_solver* s)
{
    const HostLayout& L = s->L;
    cudaStream_t st = s->stream;
    CK(s->aux.upload(L.aux, st));
    CK(s->mass.upload(L.mass, st));
    CK(s->omega.upload(L.omega, st));
    CK(s->vcloth.upload(L.vcloth, st));
    CK(s->perm_global.upload(L.perm_global, st));
    CK(s->perm_local.upload(L.perm_local, st));
    {
        std::vector<int> inv(L.ntot);
        for (int g = 0; g < L.ntot; ++g) inv[L.perm_global[g]] = g;
        CK(s->inv_global.upload(inv, st));
        CK(cudaStreamSynchronize(st));   // `inv` is a host temporary
    }
    CK(s->halo.upload(L.halo, st));
    CK(s->csr_ptr.upload(L.csr_ptr, st));
    CK(s->patches.upload(L.patches, st));
    {
        // cell records in the device format: groups of kCellGroup records,
        // 16-byte piece i of every record of a group together (pdg_layout.h)
        constexpr int P = (int)(sizeof(CellRec) / 16);
        std::vector<CellRec> dev(L.cells.size());
        const uint4* src = reinterpret_cast<const uint4*>(L.cells.data());
        uint4* dst = reinterpret_cast<uint4*>(dev.data());
        for (size_t g = 0; g < L.cells.size() / kCellGroup; ++g)
            for (int j = 0; j < kCellGroup; ++j)
                for (int i = 0; i < P; ++i)
                    dst[(g * P + i) * kCellGroup + j] = src[(g * kCellGroup + j) * P + i];
        CK(s->cells.upload(dev, st));
        CK(cudaStreamSynchronize(st));   // `dev` is a host temporary
    }
    CK(s->hinges.upload(L.hinges, st));
    CK(s->hvm.upload(L.hvm, st));
    CK(s->cinfo.upload(L.cinfo, st));
    CK(s->crt.alloc(L.ncloth));
    s->acc_stride = L.cap + 4;   // sweeps 0..cap, then r(y) and r(learned start)
    CK(s->acc.alloc((size_t)L.ncloth * s->acc_stride));
    CK(cudaMemsetAsync(s->acc.p, 0, sizeof(double) * (size_t)L.ncloth * s->acc_stride, st));
    if (s->kernel == PDG_KERNEL_RESIDENT) {
        CK(s->xch.alloc(8 * (size_t)L.ntot));
        CK(cudaMemsetAsync(s->xch.p, 0, sizeof(unsigned long long) * 8 * (size_t)L.ntot, st));
        CK(s->xch_tag.alloc(1));
        CK(cudaMemsetAsync(s->xch_tag.p, 0, sizeof(unsigned), st));
    }
    CK(s->X.alloc(L.ntot)); CK(s->V.alloc(L.ntot)); CK(s->Y.alloc(L.ntot));
    CK(s->A.alloc(L.ntot)); CK(s->B.alloc(L.ntot));
    CK(s->stage_x.alloc(3 * (size_t)L.ntot)); CK(s->stage_v.alloc(3 * (size_t)L.ntot));
    CK(s->bar.alloc(4));   // [0] arrivals, [1] generation, [2] error word
    CK(cudaMemsetAsync(s->bar.p, 0, 4 * sizeof(unsigned), st));
    CK(cudaMemsetAsync(s->crt.p, 0, sizeof(ClothRT) * L.ncloth, st));
    CK(cudaMemsetAsync(s->Y.p, 0, sizeof(float4) * L.ntot, st));
    CK(cudaMemsetAsync(s->V.p, 0, sizeof(float4) * L.ntot, st));
    // x = rest positions (ClothMesh::upload_to_gpu, src/cloth_mesh.cpp:44-55)
    std::vector<float> rest(3 * (size_t)L.ntot);
    size_t off = 0;
    for (const auto& c : s->cloths) {
        std::memcpy(rest.data() + off, c.mesh->rest.data(), sizeof(float) * c.mesh->rest.size());
        off += c.mesh->rest.size();
    }
    CK(cudaMemcpyAsync(s->stage_x.p, rest.data(), sizeof(float) * rest.size(), cudaMemcpyHostToDevice, st));
    CK(launch_scatter_state(s->stage_x.p, s->X.p, s->perm_global.p, L.ntot, st));
    CK(cudaStreamSynchronize(st));
    return PDG_OK;
}

IterArgs iter_args(pdg_solver* s)
{
    IterArgs a;
    a.patches = s->patches.p; a.halo = s->halo.p; a.cells = s->cells.p; a.hinges = s->hinges.p; a.hvm = s->hvm.p;
    a.csr_ptr = s->csr_ptr.p; a.cinfo = s->cinfo.p; a.crt = s->crt.p;
    a.omega = s->omega.p; a.omega_stride = s->L.omega_stride;
    a.Y = s->Y.p; a.buf[0] = s->A.p; a.buf[1] = s->B.p; a.ncloth = s->L.ncloth;
    a.acc = s->acc.p; a.acc_stride = s->acc_stride;
    a.have_final = s->have_final;
    a.warm_active = (s->ws && s->any_warm) ? 1 : 0;
    return a;
}

PersistArgs persist_args(pdg_solver* s)
{
    PersistArgs p;
    p.it = iter_args(s);
    p.X = s->X.p; p.Xw = s->X.p; p.V = s->V.p; p.aux = s->aux.p; p.mass = s->mass.p; p.vcloth = s->vcloth.p;
    p.warm = nullptr; p.Y = s->Y.p;
    p.n = s->L.ntot; p.npatch = s->L.npatch; p.max_iter = s->L.cap; p.have_final = s->have_final;
    p.mode = s->mode; p.bar = s->bar.p; p.err = reinterpret_cast<int*>(s->bar.p + 2);
    p.spin_budget = s->wait_budget;
    p.xch = s->xch.p;
    p.xch_tag = s->xch_tag.p;
    p.nbr_sync = s->nbr_sync;
    p.in_x = p.in_v = nullptr;
    p.out_x = p.out_v = nullptr;
    p.io_inv = s->inv_global.p;
    return p;
}

// Sweep k of the per-sweep launch structures.  after_sweep: the previous
// launch on the stream is a sweep (the streaming kernel then overlaps it).
cudaError_t launch_sweep(pdg_solver* s, const IterArgs& a, int k, int res_only, cudaStream_t st, bool after_sweep)
{
    if (s->kernel == PDG_KERNEL_STREAM) {
        s->sargs.spin_budget = s->wait_budget;
        return launch_stream(a, s->sargs, s->mode, s->nt, s->persist_grid, s->stream_smem, k, res_only, st,
                             after_sweep);
    }
    return launch_iter(a, s->mode, s->nt, s->L.npatch, s->L.smem_bytes, k, res_only, st, s->carveout);
}

// Arguments of the learned chain: the inertial chain's, with its own
// iterates, records and per-sweep sums.
IterArgs learned_chain(pdg_solver* s, const IterArgs& a)
{
    IterArgs b = a;
    b.buf[0] = s->A2.p; b.buf[1] = s->B2.p;
    b.crt = s->crt2.p; b.acc = s->acc2.p;
    return b;
}

// Sweeps each start runs before the learned start is judged (0: the start
// residuals are compared), at most the sweep cap.
int judge_sweeps(const pdg_solver* s)
{
    return (s->ws && s->any_warm) ? std::min(warm_judge_sweeps(s->ws), s->L.cap) : 0;
}

// Launches of one frame as a sequence of stream-ordered launches; the events
// (may be null) bracket the sweeps of the iteration loop.
cudaError_t enqueue_frame_launches(pdg_solver* s, cudaStream_t st, cudaEvent_t ev_sweeps0, cudaEvent_t ev_sweeps1,
                                   int* warm_rc)
{
    const HostLayout& L = s->L;
    const IterArgs a = iter_args(s);
    cudaError_t e = launch_predict(a, s->X.p, s->V.p, s->aux.p, s->mass.p, s->vcloth.p, nullptr, L.ntot, st);
    if (e != cudaSuccess) return e;
    const int K = judge_sweeps(s);
    int k0 = 0;
    if (a.warm_active) {   // learned start: predict, then judge it against the inertial start
        *warm_rc = warm_infer_enqueue(s->ws, s);
        if (*warm_rc) return cudaSuccess;
        if (K == 0) {
            e = launch_warm_select(a, s->nt, L.npatch, L.smem_bytes, s->warm.p, s->vcloth.p, L.ntot, st);
        } else {
            // both starts run K sweeps on their own chains; every cloth then
            // continues from the chain with the lower residual
            // The normaliser r(y): when no cloth always keeps the prediction,
            // every cloth's inertial chain starts from the offsets whose
            // residual it needs, so its first sweep measures it and a
            // separate evaluation is not needed.
            const IterArgs b = learned_chain(s, a);
            const bool eval_start = s->any_keep;
            e = launch_warm_chain_init(a, b, s->nt, L.npatch, L.smem_bytes, s->warm.p, s->vcloth.p, L.ntot,
                                       eval_start, st);
            if (ev_sweeps0) cudaEventRecord(ev_sweeps0, st);
            for (int k = 0; k < K && e == cudaSuccess; ++k) {
                e = launch_sweep(s, a, k, 0, st, k >= 2 || (k == 1 && eval_start));
                if (k == 0 && !eval_start && e == cudaSuccess) e = launch_warm_start_norm(a, b, st);
            }
            for (int k = 0; k < K && e == cudaSuccess; ++k) e = launch_sweep(s, b, k, 0, st, true);
            if (e == cudaSuccess) e = launch_warm_judge(a, b, K, s->vcloth.p, L.ntot, st);
            k0 = K;
        }
        if (e != cudaSuccess) return e;
    }
    if (ev_sweeps0 && k0 == 0) cudaEventRecord(ev_sweeps0, st);
    for (int k = k0; k < L.cap && e == cudaSuccess; ++k) e = launch_sweep(s, a, k, 0, st, k > k0);
    if (ev_sweeps1) cudaEventRecord(ev_sweeps1, st);
    if (e == cudaSuccess && s->have_final) e = launch_sweep(s, a, L.cap, 1, st, L.cap > k0);
    if (e == cudaSuccess) e = launch_finalize(a, s->X.p, s->V.p, s->aux.p, s->vcloth.p, L.ntot, st);
    if (e == cudaSuccess && s->ws) e = launch_keep_offset(a, s->X.p, s->aux.p, s->vcloth.p, s->dprev.p, L.ntot, st);
    return e;
}

// One frame as a sequence of stream-ordered launches.
int enqueue_frame(pdg_solver* s)
{
    int wrc = PDG_OK;
    const cudaError_t e = enqueue_frame_launches(s, s->stream, nullptr, nullptr, &wrc);
    if (wrc) return wrc;
    CK(e);
    return PDG_OK;
}

// Launches of one frame beyond the solver's own (learned start).
long long warm_launches(const pdg_solver* s)
{
    if (!s->ws) return 0;
    long long n = 1;   // the kept offset
    if (s->any_warm) {
        const int K = judge_sweeps(s);
        n += warm_kernel_count() + (K == 0 ? 4 : 3 + K + 2);
    }
    return n;
}

int build_graph(pdg_solver* s)
{
    if (s->graph) { cudaGraphExecDestroy(s->graph); s->graph = nullptr; }
    CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = enqueue_frame(s);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(s->stream, &g);
    if (rc != PDG_OK) { if (g) cudaGraphDestroy(g); return rc; }
    if (e != cudaSuccess) return set_error(PDG_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
    const cudaError_t e2 = cudaGraphInstantiate(&s->graph, g, 0);
    cudaGraphDestroy(g);
    if (e2 != cudaSuccess) return set_error(PDG_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e2));
    return PDG_OK;
}

}  // namespace

// The cloths of a solver, checked: each mesh with its own constraints, valid
// configurations, one mode.
static int collect_cloths(int n, const pdg_config* cfgs, const pdg_mesh* const* meshes,
                          const pdg_constraints* const* cons, std::vector<ClothSetup>& out)
{
    for (int i = 0; i < n; ++i) {
        if (!meshes[i] || !cons[i]) return set_error(PDG_ERR_ARG, "cloth %d: null mesh or constraints", i);
        if (cons[i]->mesh != meshes[i]->data)
            return set_error(PDG_ERR_ARG, "cloth %d: constraints were built for another mesh", i);
        const int rc = check_cfg(cfgs[i], i);
        if (rc) return rc;
        if (cfgs[i].mode != cfgs[0].mode) return set_error(PDG_ERR_ARG, "all cloths of a solver share one mode");
        ClothSetup c;
        c.mesh = meshes[i]->data;
        c.topo = cons[i]->topo;
        c.cons = cons[i]->c;
        if (c.cons.k_stretch.empty()) c.cons.k_stretch.assign(c.mesh->T, 0.f);  // no stretch data: no stretch term
        c.cfg = cfgs[i];
        out.push_back(std::move(c));
    }
    return PDG_OK;
}

int pdg::create_solver(int n, const pdg_config* cfgs, const pdg_mesh* const* meshes, const pdg_constraints* const* cons,
                       void* stream, pdg_solver** out)
{
    if (!out || n <= 0 || !cfgs || !meshes || !cons) return set_error(PDG_ERR_ARG, "solver create: bad arguments");
    std::unique_ptr<pdg_solver> s(new pdg_solver);
    {
        const int rc = collect_cloths(n, cfgs, meshes, cons, s->cloths);
        if (rc) return rc;
    }
    const pdg_config& c0 = cfgs[0];
    s->mode = c0.mode;
    s->have_final = (c0.mode == PDG_MODE_CONSISTENT) && (c0.compute_final_residual || c0.tolerance > 0.f);
    // defaults: 256-vertex patches on 256 threads, the measured best plan of
    // the streaming kernel (512-cloth batch 167.9 against 174.0 us per sweep
    // at 128 / 128, 1025x1025 57.3 against 62.6 us) and of the per-patch
    // graph kernel
    s->nt = c0.block_threads ? c0.block_threads : 256;
    if (s->nt != 128 && s->nt != 256 && s->nt != 512)
        return set_error(PDG_ERR_ARG, "block_threads must be 128, 256 or 512");
    s->patch_verts = c0.patch_verts ? c0.patch_verts : 256;
    if (c0.smem_carveout < 0 || c0.smem_carveout > 100) return set_error(PDG_ERR_ARG, "smem_carveout must be in [0, 100]");
    s->carveout = c0.smem_carveout;
    if (s->patch_verts < 16 || s->patch_verts > 4096) return set_error(PDG_ERR_ARG, "patch_verts must be in [16, 4096]");
    if (c0.kernel == PDG_KERNEL_AUTOTUNE) return autotune_create(n, cfgs, meshes, cons, stream, out);
    if (c0.kernel < PDG_KERNEL_AUTO || (c0.kernel > PDG_KERNEL_RESIDENT && c0.kernel != PDG_KERNEL_STREAM))
        return set_error(PDG_ERR_ARG, "unknown kernel");
    s->kernel = c0.kernel == PDG_KERNEL_AUTO ? PDG_KERNEL_STREAM : c0.kernel;
    for (const auto& c : s->cloths)
        s->any_warm = s->any_warm || c.cfg.init == PDG_INIT_WARMSTART || c.cfg.init == PDG_INIT_WARMSTART_KEEP;
    for (const auto& c : s->cloths) s->any_keep = s->any_keep || c.cfg.init == PDG_INIT_WARMSTART_KEEP;
    if (s->any_warm && (c0.kernel == PDG_KERNEL_PERSISTENT || c0.kernel == PDG_KERNEL_RESIDENT))
        return set_error(PDG_ERR_ARG, "the learned warm start runs with the per-sweep (graph) kernels only");

    int dev = 0;
    CK(cudaGetDevice(&dev));
    int smem_optin = 0, nsm = 0;
    CK(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    std::string err;
    if ((c0.kernel == PDG_KERNEL_AUTO && !s->any_warm) || c0.kernel == PDG_KERNEL_RESIDENT) {
        // Resident kernel: every patch co-resident, one 512-thread block per
        // SM, or (block_threads = 256) two half-size patches per SM; a block
        // is rnt compute threads and one more warp.
        const int rnt = (c0.kernel == PDG_KERNEL_RESIDENT && c0.block_threads == 256) ? 224 : 480;
        const int per_sm = 512 / (rnt + 32);
        int ntot = 0;
        for (const auto& c : s->cloths) ntot += c.mesh->N;
        int P = c0.patch_verts;
        if (!P) P = std::min(rnt, std::max(32, ((ntot + per_sm * nsm - 1) / (per_sm * nsm) + 31) / 32 * 32));
        bool ok = P <= rnt && build_layout(s->cloths, P, s->L, err);
        int variant = -1;
        if (ok) {
            variant = resident_pick(rnt);
            ok = variant >= 0 && s->L.max_nown <= rnt &&
                 s->L.smem_resident <= (size_t)std::min(smem_optin / per_sm - 8192, 216 * 1024);
            if (ok) ok = s->L.npatch <= resident_max_blocks(s->mode, variant, s->L.smem_resident);
        }
        if (ok) {
            s->kernel = PDG_KERNEL_RESIDENT;
            s->patch_verts = P;
            s->nt = rnt + 32;
            s->res_variant = variant;
            s->persist_grid = s->L.npatch;
            // fixed sweep counts: neighbour-only synchronisation between sweeps
            s->nbr_sync = 1;
            for (const auto& c : s->cloths)
                if (c.cfg.tolerance > 0.f) s->nbr_sync = 0;
        } else if (c0.kernel == PDG_KERNEL_RESIDENT) {
            return set_error(PDG_ERR_ARG, "resident kernel does not fit this problem (%d patches of %d vertices)",
                             s->L.npatch, P);
        }
    }
    for (; s->kernel != PDG_KERNEL_RESIDENT;) {
        if (!build_layout(s->cloths, s->patch_verts, s->L, err)) return set_error(PDG_ERR_ARG, "%s", err.c_str());
        if (s->kernel == PDG_KERNEL_STREAM) {
            const HostLayout& L = s->L;
            stream_layout(L.max_nown, L.max_nhalo, L.max_nlocal, L.max_vm_nslot, s->sargs, s->stream_smem);
            if (s->stream_smem + 2048 <= (size_t)smem_optin) break;
        } else if (s->L.smem_bytes + 1024 <= (size_t)std::min(smem_optin, 200 * 1024)) {
            break;
        }
        if (s->patch_verts <= 16) return set_error(PDG_ERR_ARG, "mesh too dense for the shared-memory patch layout");
        s->patch_verts /= 2;
    }
    if (stream) {
        s->stream = (cudaStream_t)stream;
    } else {
        CK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
        s->own_stream = true;
    }
    int rc = upload_all(s.get());
    if (rc) return rc;
    s->h_rt.resize(s->L.ncloth);
    s->kernels_per_frame = 4 + s->L.cap + (s->have_final ? 1 : 0);
    if (s->kernel == PDG_KERNEL_STREAM) {
        const int maxb = stream_max_blocks(s->mode, s->nt, s->stream_smem);
        if (maxb <= 0)
            return set_error(PDG_ERR_CUDA, "streaming kernel cannot be resident with %zu B of shared memory",
                             s->stream_smem);
        s->persist_grid = std::min(maxb, s->L.npatch);
        s->sargs.npatch = s->L.npatch;
        s->sargs.err = reinterpret_cast<int*>(s->bar.p + 2);
        s->sargs.spin_budget = s->wait_budget;
    }
    if (s->kernel == PDG_KERNEL_PERSISTENT) {
        int per_sm = 0;
        const int maxb = persistent_max_blocks(s->mode, s->nt, s->L.smem_bytes, &per_sm);
        if (maxb <= 0)
            return set_error(PDG_ERR_CUDA, "persistent kernel cannot be resident with %zu B of shared memory",
                             s->L.smem_bytes);
        s->persist_grid = std::min(maxb, s->L.npatch);
    }
    *out = s.release();
    return PDG_OK;
}

namespace {

int cloth_range(const pdg_solver* s, int cloth, int* vb, int* n)
{
    if (!s || cloth < 0 || cloth >= s->L.ncloth) return set_error(PDG_ERR_ARG, "cloth index out of range");
    *vb = s->L.cinfo[cloth].vbegin;
    *n = s->L.cinfo[cloth].nverts;
    return PDG_OK;
}

}  // namespace

extern "C" {

int pdg_solver_create(const pdg_config* cfg, const pdg_mesh* m, const pdg_constraints* c, void* stream,
                      pdg_solver** out)
{
    try {
        if (!cfg) return set_error(PDG_ERR_ARG, "null config");
        return pdg::create_solver(1, cfg, &m, &c, stream, out);
    } catch (const std::bad_alloc&) {
        return set_error(PDG_ERR_ALLOC, "host allocation failed");
    }
}

int pdg_solver_create_batch(int n, const pdg_config* cfgs, const pdg_mesh* const* meshes,
                            const pdg_constraints* const* cons, void* stream, pdg_solver** out)
{
    try {
        return pdg::create_solver(n, cfgs, meshes, cons, stream, out);
    } catch (const std::bad_alloc&) {
        return set_error(PDG_ERR_ALLOC, "host allocation failed");
    }
}

// One mistake planted in a built layout (for the checker's own tests): false
// if the layout offers no place for it.
static bool plant_mistake(HostLayout& L, int mistake)
{
    auto patch_with = [&](auto pred) -> int {
        for (int p = 0; p < L.npatch; ++p)
            if (pred(L.patches[p])) return p;
        return -1;
    };
    switch (mistake) {
        case 1: {   // two vertices' caller indices swapped
            const ClothInfo& c = L.cinfo[0];
            if (c.nverts < 2) return false;
            std::swap(L.perm_global[c.vbegin], L.perm_global[c.vbegin + 1]);
            return true;
        }
        case 2: {   // a halo entry repeated
            const int p = patch_with([](const PatchHdr& h) { return h.nlocal - h.nown >= 2; });
            if (p < 0) return false;
            L.halo[L.patches[p].halo_off + 1] = L.halo[L.patches[p].halo_off];
            return true;
        }
        case 3: {   // a boundary vertex moved past the published prefix
            const int p = patch_with([](const PatchHdr& h) { return h.nbnd >= 1; });
            if (p < 0) return false;
            L.patches[p].nbnd -= 1;
            return true;
        }
        case 4: {   // two records pointed at one contribution slot of a vertex they share
            auto corner = [](const CellRec& r, int k) {
                const uint32_t w = k < 2 ? r.c01 : (k < 4 ? r.c23 : r.x12);
                return (k & 1) ? w >> 16 : w & 0xffffu;
            };
            auto slot_ref = [](CellRec& r, int k) -> uint32_t& { return k < 2 ? r.vm01 : (k < 4 ? r.vm23 : r.vm45); };
            auto slot_of = [&](CellRec& r, int k) { return (k & 1) ? slot_ref(r, k) >> 16 : slot_ref(r, k) & 0xffffu; };
            for (int p = 0; p < L.npatch; ++p) {
                const PatchHdr& h = L.patches[p];
                for (int q = 0; q + 1 < h.ncell; ++q)
                    for (int q2 = q + 1; q2 < h.ncell; ++q2) {
                        CellRec& a = L.cells[h.cell_off + q];
                        CellRec& b = L.cells[h.cell_off + q2];
                        for (int ka = 0; ka < 6; ++ka)
                            for (int kb = 0; kb < 6; ++kb) {
                                if (corner(a, ka) != corner(b, kb) || slot_of(a, ka) == 0xffffu ||
                                    slot_of(b, kb) == 0xffffu)
                                    continue;
                                const uint32_t sb = slot_of(b, kb);
                                uint32_t& w = slot_ref(a, ka);
                                w = (ka & 1) ? ((w & 0xffffu) | (sb << 16)) : ((w & 0xffff0000u) | sb);
                                return true;
                            }
                    }
            }
            return false;
        }
        case 5: {   // a cell dropped
            const int p = patch_with([](const PatchHdr& h) { return h.ncell >= 2; });
            if (p < 0) return false;
            L.patches[p].ncell -= 1;
            if (L.patches[p].ncell_a > L.patches[p].ncell) L.patches[p].ncell_a = L.patches[p].ncell;
            return true;
        }
        case 6: {   // a halo entry out of range
            const int p = patch_with([](const PatchHdr& h) { return h.nlocal - h.nown >= 1; });
            if (p < 0) return false;
            L.halo[L.patches[p].halo_off] = L.ntot + 5;
            return true;
        }
    }
    return false;
}

static int layout_check_impl(int n, const pdg_config* cfgs, const pdg_mesh* const* meshes,
                             const pdg_constraints* const* cons, int patch_verts, int mistake, pdg_layout_info* info)
{
    try {
        if (n <= 0 || !cfgs || !meshes || !cons || !info) return set_error(PDG_ERR_ARG, "pdg_layout_check: bad arguments");
        if (patch_verts < 16 || patch_verts > 4096) return set_error(PDG_ERR_ARG, "patch_verts must be in [16, 4096]");
        std::vector<ClothSetup> cl;
        int rc = collect_cloths(n, cfgs, meshes, cons, cl);
        if (rc) return rc;
        HostLayout L;
        std::string err;
        if (!build_layout(cl, patch_verts, L, err)) return set_error(PDG_ERR_ARG, "%s", err.c_str());
        *info = pdg_layout_info{};
        info->vertices = L.ntot;
        info->patches = L.npatch;
        info->max_owned = L.max_nown;
        info->max_local = L.max_nlocal;
        for (const PatchHdr& h : L.patches) {
            info->halo_total += h.nlocal - h.nown;
            info->boundary_total += h.nbnd;
            info->phase_a_cells += h.ncell_a;
        }
        info->cells = 0;
        for (const PatchHdr& h : L.patches) info->cells += h.ncell;
        info->lone_hinges = (long long)L.hinges.size();
        info->smem_resident = (long long)L.smem_resident;
        if (mistake && !plant_mistake(L, mistake))
            return set_error(PDG_ERR_ARG, "pdg_layout_check_planted: no place for mistake %d in this layout", mistake);
        err = check_layout(cl, L);
        if (!err.empty()) return set_error(PDG_ERR_STATE, "layout check: %s", err.c_str());
        return PDG_OK;
    } catch (const std::bad_alloc&) {
        return set_error(PDG_ERR_ALLOC, "host allocation failed");
    }
}

int pdg_layout_check(int n, const pdg_config* cfgs, const pdg_mesh* const* meshes, const pdg_constraints* const* cons,
                     int patch_verts, pdg_layout_info* info)
{
    return layout_check_impl(n, cfgs, meshes, cons, patch_verts, 0, info);
}

int pdg_layout_check_planted(int n, const pdg_config* cfgs, const pdg_mesh* const* meshes,
                             const pdg_constraints* const* cons, int patch_verts, int mistake, pdg_layout_info* info)
{
    if (mistake < 1 || mistake > 6) return set_error(PDG_ERR_ARG, "pdg_layout_check_planted: mistake must be 1..6");
    return layout_check_impl(n, cfgs, meshes, cons, patch_verts, mistake, info);
}

int pdg_solver_num_cloths(const pdg_solver* s, int* n)
{
    if (!s || !n) return set_error(PDG_ERR_ARG, "bad arguments");
    *n = s->L.ncloth;
    return PDG_OK;
}

int pdg_solver_cloth_counts(const pdg_solver* s, int cloth, int* N, int* T)
{
    int vb = 0, n = 0;
    const int rc = cloth_range(s, cloth, &vb, &n);
    if (rc) return rc;
    if (N) *N = n;
    if (T) *T = s->cloths[cloth].mesh->T;
    return PDG_OK;
}

// Reads and clears the error word of the bounded waits (stream synchronised).
static int take_wait_error(pdg_solver* s)
{
    int e = 0;
    CK(cudaMemcpyAsync(&e, s->bar.p + 2, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    if (!e) return PDG_OK;
    CK(cudaMemsetAsync(s->bar.p + 2, 0, sizeof(int), s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return set_error(PDG_ERR_TIMEOUT, "bounded wait ran out (%s)",
                     e == 1 ? "grid barrier" : e == 2 ? "resident grid barrier" : "neighbour exchange");
}

// Caller state moved by the resident frame launch itself: inputs read by the
// first frame, outputs written by the last (device or mapped host pointers).
struct FrameIO {
    const float* in_x;
    const float* in_v;
    float* out_x;
    float* out_v;
};

// `nframes` frames, stream-ordered; `io` only with the resident kernel.
static int enqueue_frames(pdg_solver* s, int nframes, const FrameIO* io)
{
    for (int f = 0; f < nframes; ++f) {
        if (s->kernel == PDG_KERNEL_PERSISTENT || s->kernel == PDG_KERNEL_RESIDENT) {
            // barrier counter and generation start clean every frame; the
            // error word stays set until it is reported, and a kernel that
            // finds it set leaves at its first barrier
            CK(cudaMemsetAsync(s->bar.p, 0, 2 * sizeof(unsigned), s->stream));
            PersistArgs p = persist_args(s);
            if (io && f == 0) { p.in_x = io->in_x; p.in_v = io->in_v; }
            if (io && f == nframes - 1) { p.out_x = io->out_x; p.out_v = io->out_v; }
            if (s->kernel == PDG_KERNEL_PERSISTENT)
                CK(launch_persistent(p, s->nt, s->persist_grid, s->L.smem_bytes, s->stream));
            else
                CK(launch_resident(p, s->res_variant, s->persist_grid, s->L.smem_resident, s->stream));
            s->launches += 1;
        } else {
            if (!s->graph) {
                const int rc = build_graph(s);
                if (rc) return rc;
            }
            CK(cudaGraphLaunch(s->graph, s->stream));
            s->launches += s->kernels_per_frame + warm_launches(s);
        }
    }
    return PDG_OK;
}

int pdg_solver_step(pdg_solver* s, int nframes, pdg_frame_stats* stats)
{
    if (!s || nframes < 0) return set_error(PDG_ERR_ARG, "pdg_solver_step: bad arguments");
    const int rc = enqueue_frames(s, nframes, nullptr);
    if (rc) return rc;
    if (stats) {
        CK(cudaMemcpyAsync(s->h_rt.data(), s->crt.p, sizeof(ClothRT) * s->L.ncloth, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        if (s->kernel != PDG_KERNEL_GRAPH) {   // bounded waits of the one-launch and streaming kernels
            const int rc = take_wait_error(s);
            if (rc) return rc;
        }
        for (int c = 0; c < s->L.ncloth; ++c) {
            const ClothRT& r = s->h_rt[c];
            const ClothInfo& ci = s->L.cinfo[c];
            pdg_frame_stats& o = stats[c];
            o.iterations = r.used;
            o.warm_start_used = r.warm;
            o.status = r.status;
            o.res_inertial = std::sqrt(std::max(0.0, r.res_y2));
            o.res_initial = std::sqrt(std::max(0.0, r.res0_2));
            o.res_final = r.resf_2 >= 0.0 ? std::sqrt(r.resf_2) : (std::isnan(r.resf_2) ? NAN : -1.0);
            o.rel_residual = (o.res_final >= 0.0 && o.res_inertial > 0.0) ? o.res_final / o.res_inertial
                             : (o.res_final == 0.0 ? 0.0 : -1.0);
            o.converged = (r.status == 0 && ci.tol > 0.f && o.res_final >= 0.0 &&
                           o.res_final <= (double)ci.tol * o.res_inertial) ? 1 : 0;
        }
    }
    return PDG_OK;
}

int pdg_solver_reset(pdg_solver* s)
{
    // The Chebyshev weights restart every frame; nothing persists between frames.
    if (!s) return set_error(PDG_ERR_ARG, "null solver");
    return PDG_OK;
}

// State copies between caller order (AoS xyz) and the solver's float4
// arrays; host pointers go through the device staging buffers.  Both arrays
// move in one scatter or gather launch.  `sync` = 0 leaves the copies
// enqueued on the solver's stream.
static int put_state(pdg_solver* s, int vb, int n, const float* x, const float* v, int on_device, bool whole)
{
    if (!x && !v) return PDG_OK;
    const int* perm = whole ? s->perm_global.p : s->perm_local.p + vb;
    if (!on_device) {
        if (x) CK(cudaMemcpyAsync(s->stage_x.p, x, sizeof(float) * 3 * (size_t)n, cudaMemcpyHostToDevice, s->stream));
        if (v) CK(cudaMemcpyAsync(s->stage_v.p, v, sizeof(float) * 3 * (size_t)n, cudaMemcpyHostToDevice, s->stream));
        x = x ? s->stage_x.p : nullptr;
        v = v ? s->stage_v.p : nullptr;
    }
    CK(launch_scatter_state(x, s->X.p + vb, perm, n, s->stream, v, s->V.p + vb, s->dprev.p ? s->dprev.p + vb : nullptr));
    return PDG_OK;
}

static int take_state(pdg_solver* s, int vb, int n, float* x, float* v, int on_device, bool whole)
{
    if (!x && !v) return PDG_OK;
    const int* perm = whole ? s->perm_global.p : s->perm_local.p + vb;
    float* dx = (x && !on_device) ? s->stage_x.p : x;
    float* dv = (v && !on_device) ? s->stage_v.p : v;
    CK(launch_gather_state(s->X.p + vb, dx, perm, n, s->stream, s->V.p + vb, dv));
    if (!on_device) {
        if (x) CK(cudaMemcpyAsync(x, dx, sizeof(float) * 3 * (size_t)n, cudaMemcpyDeviceToHost, s->stream));
        if (v) CK(cudaMemcpyAsync(v, dv, sizeof(float) * 3 * (size_t)n, cudaMemcpyDeviceToHost, s->stream));
    }
    return PDG_OK;
}

static int set_state_range(pdg_solver* s, int vb, int n, const float* x, const float* v, int on_device, bool whole)
{
    const int rc = put_state(s, vb, n, x, v, on_device, whole);
    if (rc) return rc;
    if (!on_device) CK(cudaStreamSynchronize(s->stream));
    return PDG_OK;
}

static int get_state_range(pdg_solver* s, int vb, int n, float* x, float* v, int on_device, bool whole)
{
    const int rc = take_state(s, vb, n, x, v, on_device, whole);
    if (rc) return rc;
    if (!on_device) CK(cudaStreamSynchronize(s->stream));
    return PDG_OK;
}

int pdg_solver_set_state(pdg_solver* s, int cloth, const float* x, const float* v, int on_device)
{
    int vb = 0, n = 0;
    const int rc = cloth_range(s, cloth, &vb, &n);
    return rc ? rc : set_state_range(s, vb, n, x, v, on_device, false);
}

int pdg_solver_get_state(pdg_solver* s, int cloth, float* x, float* v, int on_device)
{
    int vb = 0, n = 0;
    const int rc = cloth_range(s, cloth, &vb, &n);
    return rc ? rc : get_state_range(s, vb, n, x, v, on_device, false);
}

int pdg_solver_set_state_all(pdg_solver* s, const float* x, const float* v, int on_device)
{
    if (!s) return set_error(PDG_ERR_ARG, "null solver");
    return set_state_range(s, 0, s->L.ntot, x, v, on_device, true);
}

int pdg_solver_get_state_all(pdg_solver* s, float* x, float* v, int on_device)
{
    if (!s) return set_error(PDG_ERR_ARG, "null solver");
    return get_state_range(s, 0, s->L.ntot, x, v, on_device, true);
}

// Device address of a host buffer that kernels may read and write in place
// (page-locked and mapped into the device's address space), else nullptr.
static void* mapped_host(const void* p)
{
    if (!p) return nullptr;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

int pdg_solver_step_host(pdg_solver* s, int nframes, const float* x_in, const float* v_in, float* x_out,
                         float* v_out, pdg_frame_stats* stats)
{
    if (!s || nframes < 0) return set_error(PDG_ERR_ARG, "pdg_solver_step_host: bad arguments");
    // Page-locked caller buffers are read and written in place; pageable ones
    // go through the device staging buffers.
    const int n = s->L.ntot;
    const size_t bytes = sizeof(float) * 3 * (size_t)n;
    if (s->kernel == PDG_KERNEL_RESIDENT && nframes > 0 && resident_moves_state(s->mode)) {
        // The frame launch itself reads the inputs before its prediction and
        // writes the outputs after its last sweep: no copy launches around it.
        FrameIO io{static_cast<const float*>(mapped_host(x_in)), static_cast<const float*>(mapped_host(v_in)),
                   static_cast<float*>(mapped_host(x_out)), static_cast<float*>(mapped_host(v_out))};
        if (x_in && !io.in_x) {
            CK(cudaMemcpyAsync(s->stage_x.p, x_in, bytes, cudaMemcpyHostToDevice, s->stream));
            io.in_x = s->stage_x.p;
        }
        if (v_in && !io.in_v) {
            CK(cudaMemcpyAsync(s->stage_v.p, v_in, bytes, cudaMemcpyHostToDevice, s->stream));
            io.in_v = s->stage_v.p;
        }
        // a staged output lands in the staging buffer after the input has
        // been read from it (the input is read by the first frame, before
        // its first grid barrier; the output is written by the last)
        if (x_out && !io.out_x) io.out_x = s->stage_x.p;
        if (v_out && !io.out_v) io.out_v = s->stage_v.p;
        const int rc = enqueue_frames(s, nframes, &io);
        if (rc) return rc;
        if (x_out && io.out_x == s->stage_x.p)
            CK(cudaMemcpyAsync(x_out, io.out_x, bytes, cudaMemcpyDeviceToHost, s->stream));
        if (v_out && io.out_v == s->stage_v.p)
            CK(cudaMemcpyAsync(v_out, io.out_v, bytes, cudaMemcpyDeviceToHost, s->stream));
        if (stats) return pdg_solver_step(s, 0, stats);
        CK(cudaStreamSynchronize(s->stream));
        return PDG_OK;
    }
    // Other plans: copy kernels in caller order (host memory is walked
    // contiguously) around the frames.  A state of at least kDmaStateBytes
    // per array is moved by DMA into the staging buffers first.  On the
    // 3.3 M-vertex batch that took 0.73 ms per frame against 1.03 ms for the
    // copy kernels reading page-locked host memory in place.  Smaller
    // states are read and written in place, which needs no DMA.
    constexpr size_t kDmaStateBytes = 4u << 20;
    const bool dma = bytes >= kDmaStateBytes;
    if (x_in || v_in) {
        const float* dx = dma ? nullptr : static_cast<const float*>(mapped_host(x_in));
        const float* dv = dma ? nullptr : static_cast<const float*>(mapped_host(v_in));
        if (x_in && !dx) {
            CK(cudaMemcpyAsync(s->stage_x.p, x_in, bytes, cudaMemcpyHostToDevice, s->stream));
            dx = s->stage_x.p;
        }
        if (v_in && !dv) {
            CK(cudaMemcpyAsync(s->stage_v.p, v_in, bytes, cudaMemcpyHostToDevice, s->stream));
            dv = s->stage_v.p;
        }
        CK(launch_put_state(dx, dv, s->X.p, s->V.p, s->inv_global.p, n, s->stream, s->dprev.p));
    }
    // the frames, then the download: all stream-ordered behind the upload
    int rc = pdg_solver_step(s, nframes, nullptr);
    if (rc) return rc;
    if (x_out || v_out) {
        float* mx = dma ? nullptr : static_cast<float*>(mapped_host(x_out));
        float* mv = dma ? nullptr : static_cast<float*>(mapped_host(v_out));
        float* dx = x_out ? (mx ? mx : s->stage_x.p) : nullptr;
        float* dv = v_out ? (mv ? mv : s->stage_v.p) : nullptr;
        CK(launch_take_state(s->X.p, s->V.p, dx, dv, s->inv_global.p, n, s->stream));
        if (x_out && !mx) CK(cudaMemcpyAsync(x_out, dx, bytes, cudaMemcpyDeviceToHost, s->stream));
        if (v_out && !mv) CK(cudaMemcpyAsync(v_out, dv, bytes, cudaMemcpyDeviceToHost, s->stream));
    }
    if (stats) return pdg_solver_step(s, 0, stats);   // reads the last frame's records (synchronises)
    CK(cudaStreamSynchronize(s->stream));
    return PDG_OK;
}

int pdg_solver_set_tolerance(pdg_solver* s, int cloth, float tolerance)
{
    if (!s || !(tolerance >= 0.f) || !std::isfinite(tolerance))
        return set_error(PDG_ERR_ARG, "pdg_solver_set_tolerance: tolerance must be finite and >= 0");
    if (cloth < -1 || cloth >= s->L.ncloth) return set_error(PDG_ERR_ARG, "pdg_solver_set_tolerance: bad cloth");
    const int c0 = cloth < 0 ? 0 : cloth, c1 = cloth < 0 ? s->L.ncloth : cloth + 1;
    for (int c = c0; c < c1; ++c) {
        s->L.cinfo[c].tol = tolerance;
        s->cloths[c].cfg.tolerance = tolerance;
    }
    CK(cudaMemcpyAsync(s->cinfo.p, s->L.cinfo.data(), sizeof(ClothInfo) * s->L.cinfo.size(), cudaMemcpyHostToDevice,
                       s->stream));
    CK(cudaStreamSynchronize(s->stream));
    // the launch plan's choices that depend on the tolerance (as at creation)
    if (s->kernel == PDG_KERNEL_RESIDENT) {
        s->nbr_sync = 1;
        for (const auto& c : s->cloths)
            if (c.cfg.tolerance > 0.f) s->nbr_sync = 0;
    }
    const pdg_config& f = s->cloths[0].cfg;
    const int hf = (s->mode == PDG_MODE_CONSISTENT) && (f.compute_final_residual || f.tolerance > 0.f);
    if (hf != s->have_final) {
        s->have_final = hf;
        s->kernels_per_frame = 4 + s->L.cap + (hf ? 1 : 0);
        if (s->graph) { cudaGraphExecDestroy(s->graph); s->graph = nullptr; }
    }
    return PDG_OK;
}

int pdg_solver_set_pins(pdg_solver* s, int cloth, const int* idx, int P, const float* targets)
{
    int vb = 0, n = 0;
    int rc = cloth_range(s, cloth, &vb, &n);
    if (rc) return rc;
    if (P < 0 || (P > 0 && !idx)) return set_error(PDG_ERR_ARG, "pdg_solver_set_pins: bad pin list");
    ClothSetup& c = s->cloths[cloth];
    const int N = c.mesh->N;
    std::vector<char> seen(N, 0);
    for (int q = 0; q < P; ++q) {
        if (idx[q] < 0 || idx[q] >= N) return set_error(PDG_ERR_ARG, "pdg_solver_set_pins: pin %d out of range", idx[q]);
        if (seen[idx[q]]++) return set_error(PDG_ERR_ARG, "pdg_solver_set_pins: pin %d repeated", idx[q]);
        if (targets && (!std::isfinite(targets[3 * q]) || !std::isfinite(targets[3 * q + 1]) ||
                        !std::isfinite(targets[3 * q + 2])))
            return set_error(PDG_ERR_ARG, "pdg_solver_set_pins: non-finite target");
    }
    c.cons.pins.assign(idx, idx + P);
    c.cons.targets.resize(3 * (size_t)P);
    for (int q = 0; q < P; ++q)
        for (int d = 0; d < 3; ++d)
            c.cons.targets[3 * q + d] = targets ? targets[3 * q + d] : c.mesh->rest[3 * (size_t)idx[q] + d];
    // a vertex's record: its target with w = -1 when pinned, else its
    // inverse Jacobi diagonal (as the layout builds it)
    std::vector<float> diag;
    jacobi_diag(*c.mesh, c.cons, c.cfg.dt, diag);
    std::vector<int> slot(N, -1);
    for (int q = 0; q < P; ++q) slot[idx[q]] = q;
    for (int g = vb; g < vb + n; ++g) {
        const int o = s->L.perm_local[g];
        float4& a = s->L.aux[g];
        if (slot[o] >= 0) {
            const int q = slot[o];
            a = make_float4(c.cons.targets[3 * q], c.cons.targets[3 * q + 1], c.cons.targets[3 * q + 2], -1.f);
        } else {
            a = make_float4(0.f, 0.f, 0.f, diag[o] > 1e-10f ? 1.0f / diag[o] : 0.f);
        }
    }
    CK(cudaMemcpyAsync(s->aux.p + vb, s->L.aux.data() + vb, sizeof(float4) * (size_t)n, cudaMemcpyHostToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return PDG_OK;
}

int pdg_solver_set_pin_targets(pdg_solver* s, int cloth, const float* targets)
{
    int vb = 0, n = 0;
    int rc = cloth_range(s, cloth, &vb, &n);
    if (rc) return rc;
    if (!targets) return set_error(PDG_ERR_ARG, "null targets");
    ClothSetup& c = s->cloths[cloth];
    const int P = (int)c.cons.pins.size();
    for (int i = 0; i < 3 * P; ++i)
        if (!std::isfinite(targets[i])) return set_error(PDG_ERR_ARG, "non-finite pin target");
    std::memcpy(c.cons.targets.data(), targets, sizeof(float) * 3 * (size_t)P);
    for (int g = vb; g < vb + n; ++g) {
        float4& a = s->L.aux[g];
        if (a.w >= 0.f) continue;
        const int o = s->L.perm_local[g];
        for (int q = 0; q < P; ++q)
            if (c.cons.pins[q] == o) { a.x = targets[3 * q]; a.y = targets[3 * q + 1]; a.z = targets[3 * q + 2]; }
    }
    CK(cudaMemcpyAsync(s->aux.p + vb, s->L.aux.data() + vb, sizeof(float4) * (size_t)n, cudaMemcpyHostToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return PDG_OK;
}

int pdg_solver_get_prediction(pdg_solver* s, int cloth, float* y)
{
    int vb = 0, n = 0;
    const int rc = cloth_range(s, cloth, &vb, &n);
    if (rc) return rc;
    if (!y) return set_error(PDG_ERR_ARG, "null output");
    CK(launch_gather_state(s->Y.p + vb, s->stage_x.p, s->perm_local.p + vb, n, s->stream));
    CK(cudaMemcpyAsync(y, s->stage_x.p, sizeof(float) * 3 * (size_t)n, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return PDG_OK;
}

int pdg_solver_time_frames(pdg_solver* s, int nframes, float* frame_ms, float* sweep_ms)
{
    if (!s || nframes <= 0) return set_error(PDG_ERR_ARG, "pdg_solver_time_frames: bad arguments");
    cudaEvent_t e[4];
    for (auto& ev : e) CK(cudaEventCreate(&ev));
    const HostLayout& L = s->L;
    cudaStream_t st = s->stream;
    double tf = 0.0, ts = 0.0;
    int rc = PDG_OK;
    for (int f = 0; f < nframes && rc == PDG_OK; ++f) {
        cudaEventRecord(e[0], st);
        if (s->kernel == PDG_KERNEL_PERSISTENT || s->kernel == PDG_KERNEL_RESIDENT) {
            cudaError_t err = cudaMemsetAsync(s->bar.p, 0, 2 * sizeof(unsigned), st);
            cudaEventRecord(e[0], st);   // the frame's events bracket the launch only
            const PersistArgs p = persist_args(s);
            if (err == cudaSuccess)
                err = s->kernel == PDG_KERNEL_RESIDENT
                          ? launch_resident(p, s->res_variant, s->persist_grid, L.smem_resident, st)
                          : launch_persistent(p, s->nt, s->persist_grid, L.smem_bytes, st);
            if (err != cudaSuccess) rc = set_error(PDG_ERR_CUDA, "persistent launch: %s", cudaGetErrorString(err));
            s->launches += 1;
            cudaEventRecord(e[1], st); cudaEventRecord(e[2], st);
        } else {
            int wrc = PDG_OK;
            const cudaError_t err = enqueue_frame_launches(s, st, e[1], e[2], &wrc);
            if (wrc) { rc = wrc; break; }
            if (err != cudaSuccess) rc = set_error(PDG_ERR_CUDA, "frame launch: %s", cudaGetErrorString(err));
            s->launches += s->kernels_per_frame + warm_launches(s);
        }
        cudaEventRecord(e[3], st);
        cudaError_t se = cudaEventSynchronize(e[3]);
        if (se != cudaSuccess) { rc = set_error(PDG_ERR_CUDA, "frame: %s", cudaGetErrorString(se)); break; }
        float a = 0.f, b = 0.f;
        cudaEventElapsedTime(&a, e[0], e[3]);
        cudaEventElapsedTime(&b, e[1], e[2]);
        tf += a;
        ts += (s->kernel == PDG_KERNEL_PERSISTENT || s->kernel == PDG_KERNEL_RESIDENT) ? a : b;
    }
    for (auto& ev : e) cudaEventDestroy(ev);
    if (rc) return rc;
    if (s->kernel != PDG_KERNEL_GRAPH) {
        rc = take_wait_error(s);
        if (rc) return rc;
    }
    if (frame_ms) *frame_ms = (float)(tf / nframes);
    const bool one_launch = s->kernel == PDG_KERNEL_PERSISTENT || s->kernel == PDG_KERNEL_RESIDENT;
    const int sweeps = std::max(1, L.cap + (one_launch && s->have_final ? 1 : 0));
    if (sweep_ms) *sweep_ms = (float)(ts / nframes / sweeps);
    return PDG_OK;
}

int pdg_solver_set_wait_budget(pdg_solver* s, long long cycles)
{
    if (!s || cycles < 0) return set_error(PDG_ERR_ARG, "pdg_solver_set_wait_budget: bad arguments");
    s->wait_budget = cycles;
    // the streaming kernel's budget is a launch argument inside the graph
    if (s->graph) { cudaGraphExecDestroy(s->graph); s->graph = nullptr; }
    return PDG_OK;
}

int pdg_solver_set_frame_tag(pdg_solver* s, unsigned long long tag)
{
    if (!s || tag > 0xffffffffULL) return set_error(PDG_ERR_ARG, "pdg_solver_set_frame_tag: bad arguments");
    if (!s->xch_tag.p) return PDG_OK;   // not the resident kernel
    const unsigned t = (unsigned)tag;
    CK(cudaMemcpyAsync(s->xch_tag.p, &t, sizeof(unsigned), cudaMemcpyHostToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));   // `t` is a host temporary
    return PDG_OK;
}

int pdg_solver_launch_count(const pdg_solver* s, long long* n)
{
    if (!s || !n) return set_error(PDG_ERR_ARG, "bad arguments");
    *n = s->launches;
    return PDG_OK;
}

int pdg_solver_stream(const pdg_solver* s, void** stream)
{
    if (!s || !stream) return set_error(PDG_ERR_ARG, "bad arguments");
    *stream = (void*)s->stream;
    return PDG_OK;
}

int pdg_solver_launch_info(const pdg_solver* s, int* kernel, int* patch_verts, int* block_threads, int* npatches)
{
    if (!s) return set_error(PDG_ERR_ARG, "null solver");
    if (kernel) *kernel = s->kernel;
    if (patch_verts) *patch_verts = s->patch_verts;
    if (block_threads) *block_threads = s->nt;
    if (npatches) *npatches = s->L.npatch;
    return PDG_OK;
}

void pdg_solver_destroy(pdg_solver* s) { delete s; }

int pdg_apply_pins(float* d_pos, float* d_vel, const int* d_idx, const float* d_target, int P, void* stream)
{
    if (P < 0 || (P > 0 && (!d_pos || !d_idx || !d_target))) return set_error(PDG_ERR_ARG, "pdg_apply_pins: bad arguments");
    CK(launch_apply_pins(d_pos, d_vel, d_idx, d_target, P, (cudaStream_t)stream));
    return PDG_OK;
}

}  // extern "C"
