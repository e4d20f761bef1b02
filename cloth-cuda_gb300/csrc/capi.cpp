// C ABI of the PD cloth library: mesh, topology, constraints and solver
// handles (include/pdg.h).  Errors are returned as status codes with a
// thread-local message; nothing here exits the process (the reference's
// CUDA_CHECK exits, src/utils/cuda_helper.h:9-17).
#include "pdg_solver.h"

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>

namespace pdg {

static thread_local std::string g_last_error;

int set_error(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

}  // namespace pdg

using namespace pdg;

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return set_error(e_ == cudaErrorMemoryAllocation ? PDG_ERR_ALLOC : PDG_ERR_CUDA,  \
                             "%s failed: %s", #call, cudaGetErrorString(e_));                 \
    } while (0)

#define GUARD_BEGIN try {
#define GUARD_END                                                                             \
    }                                                                                         \
    catch (const std::bad_alloc&) { return set_error(PDG_ERR_ALLOC, "host allocation failed"); } \
    catch (const std::exception& ex) { return set_error(PDG_ERR_ARG, "%s", ex.what()); }

extern "C" {

const char* pdg_last_error_string(void) { return g_last_error.c_str(); }
const char* pdg_version(void) { return "cloth-pdg 0.1 (sm_103a)"; }

int pdg_config_default(pdg_config* c)
{
    if (!c) return set_error(PDG_ERR_ARG, "null config");
    std::memset(c, 0, sizeof(*c));
    c->max_iterations = 50;
    c->tolerance = 0.0f;   // the reference declares 1e-4 but never reads it: fixed iterations
    c->use_chebyshev = 1;
    c->rho = 0.9f;
    c->gravity = -9.8f;
    c->dt = 0.01f;
    c->stretch_stiffness = 1.0f;
    c->bend_stiffness = 0.0f;
    c->damping = 0.0f;
    c->cheb_delay = 1;
    c->gamma = 1.0f;
    c->mode = PDG_MODE_CONSISTENT;
    c->init = PDG_INIT_INERTIAL;
    c->kernel = PDG_KERNEL_AUTO;
    c->patch_verts = 0;
    c->block_threads = 0;
    c->compute_final_residual = 1;
    c->smem_carveout = 0;
    return PDG_OK;
}

// ------------------------------------------------------------------ mesh
static int finish_mesh(std::shared_ptr<MeshData> d, pdg_mesh** out)
{
    precompute_rest_state(*d);
    pdg_mesh* m = new pdg_mesh;
    m->data = d;
    *out = m;
    return PDG_OK;
}

int pdg_mesh_create(const float* rest_xyz, int N, const int* tris, int T, float density, pdg_mesh** out)
{
    GUARD_BEGIN
    if (!out || !rest_xyz || !tris || N <= 0 || T <= 0) return set_error(PDG_ERR_ARG, "pdg_mesh_create: bad arguments");
    if (!(density > 0.f)) return set_error(PDG_ERR_ARG, "pdg_mesh_create: density must be > 0");
    for (int i = 0; i < 3 * T; ++i)
        if (tris[i] < 0 || tris[i] >= N) return set_error(PDG_ERR_ARG, "pdg_mesh_create: triangle index %d out of range", tris[i]);
    for (int i = 0; i < 3 * N; ++i)
        if (!std::isfinite(rest_xyz[i])) return set_error(PDG_ERR_ARG, "pdg_mesh_create: non-finite rest position");
    auto d = std::make_shared<MeshData>();
    d->N = N; d->T = T; d->density = density;
    d->rest.assign(rest_xyz, rest_xyz + 3 * (size_t)N);
    d->tris.assign(tris, tris + 3 * (size_t)T);
    return finish_mesh(d, out);
    GUARD_END
}

int pdg_mesh_generate(int nrows, int ncols, float size, int type, float density, pdg_mesh** out)
{
    GUARD_BEGIN
    if (!out || nrows < 2 || ncols < 2 || type < 0 || type > 3 || !(size > 0.f) || !(density > 0.f))
        return set_error(PDG_ERR_ARG, "pdg_mesh_generate: need nrows, ncols >= 2, type 0..3, size > 0");
    auto d = std::make_shared<MeshData>();
    generate_grid(nrows, ncols, size, type, d->rest, d->tris);
    d->N = (int)(d->rest.size() / 3); d->T = (int)(d->tris.size() / 3); d->density = density;
    return finish_mesh(d, out);
    GUARD_END
}

int pdg_mesh_generate_hanging(int nrows, int ncols, float side, int type, float jitter,
                              unsigned long long seed, float density, pdg_mesh** out)
{
    GUARD_BEGIN
    if (!out || nrows < 2 || ncols < 2 || type < 0 || type > 3 || !(side > 0.f) || !(density > 0.f) || jitter < 0.f)
        return set_error(PDG_ERR_ARG, "pdg_mesh_generate_hanging: bad arguments");
    auto d = std::make_shared<MeshData>();
    std::vector<float> grid;
    const float cell = side / (float)(std::max(nrows, ncols) - 1);
    generate_grid(nrows, ncols, cell, type, grid, d->tris);
    const int N = (int)(grid.size() / 3);
    d->rest.resize(grid.size());
    uint64_t s = seed;
    for (int i = 0; i < N; ++i) {
        d->rest[3 * i + 0] = grid[3 * i + 0];
        d->rest[3 * i + 1] = -grid[3 * i + 2];   // reference z (row) -> -y: row 0 on top
        d->rest[3 * i + 2] = jitter > 0.f ? (float)(gaussian(s) * jitter) : 0.f;
    }
    d->N = N; d->T = (int)(d->tris.size() / 3); d->density = density;
    return finish_mesh(d, out);
    GUARD_END
}

int pdg_mesh_load_obj(const char* path, float density, pdg_mesh** out)
{
    GUARD_BEGIN
    if (!out || !path || !(density > 0.f)) return set_error(PDG_ERR_ARG, "pdg_mesh_load_obj: bad arguments");
    auto d = std::make_shared<MeshData>();
    std::string err;
    if (!load_obj(path, d->rest, d->tris, err)) return set_error(PDG_ERR_IO, "pdg_mesh_load_obj: %s", err.c_str());
    d->N = (int)(d->rest.size() / 3); d->T = (int)(d->tris.size() / 3); d->density = density;
    return finish_mesh(d, out);
    GUARD_END
}

int pdg_mesh_counts(const pdg_mesh* m, int* N, int* T)
{
    if (!m) return set_error(PDG_ERR_ARG, "null mesh");
    if (N) *N = m->data->N;
    if (T) *T = m->data->T;
    return PDG_OK;
}

int pdg_mesh_get(const pdg_mesh* m, float* rest_xyz, int* tris, float* Dm_inv, float* area, float* mass, float* dFdx)
{
    if (!m) return set_error(PDG_ERR_ARG, "null mesh");
    const MeshData& d = *m->data;
    if (rest_xyz) std::memcpy(rest_xyz, d.rest.data(), sizeof(float) * d.rest.size());
    if (tris) std::memcpy(tris, d.tris.data(), sizeof(int) * d.tris.size());
    if (Dm_inv) std::memcpy(Dm_inv, d.Dm_inv.data(), sizeof(float) * d.Dm_inv.size());
    if (area) std::memcpy(area, d.area.data(), sizeof(float) * d.area.size());
    if (mass) std::memcpy(mass, d.mass.data(), sizeof(float) * d.mass.size());
    if (dFdx)
        for (int t = 0; t < d.T; ++t) {
            // dF/dx = kron(Dm_inv^T [[-1,1,0],[-1,0,1]], I3) (src/cloth_mesh.cpp:189-204)
            const float* G = &d.Dm_inv[4 * t];
            const float D[2][3] = {{-(G[0] + G[1]), G[0], G[1]}, {-(G[2] + G[3]), G[2], G[3]}};
            float* M = dFdx + 54 * (size_t)t;
            std::memset(M, 0, sizeof(float) * 54);
            for (int r = 0; r < 2; ++r)
                for (int v = 0; v < 3; ++v)
                    for (int k = 0; k < 3; ++k) M[(3 * r + k) * 9 + 3 * v + k] = D[r][v];
        }
    return PDG_OK;
}

void pdg_mesh_destroy(pdg_mesh* m) { delete m; }

// -------------------------------------------------------------- topology
static const Topology& topo_of(const pdg_mesh* m)
{
    if (!m->topo) {
        auto t = std::make_shared<Topology>();
        build_topology(*m->data, *t);
        const_cast<pdg_mesh*>(m)->topo = t;
    }
    return *m->topo;
}

int pdg_topology_counts(const pdg_mesh* m, int* num_edges, int* num_inner)
{
    GUARD_BEGIN
    if (!m) return set_error(PDG_ERR_ARG, "null mesh");
    const Topology& t = topo_of(m);
    if (num_edges) *num_edges = (int)(t.edges.size() / 4);
    if (num_inner) *num_inner = t.num_inner;
    return PDG_OK;
    GUARD_END
}

int pdg_topology_get(const pdg_mesh* m, int* edges, float* rest_len, int* vt_ptr, int* vt, int* tri_tri)
{
    GUARD_BEGIN
    if (!m) return set_error(PDG_ERR_ARG, "null mesh");
    const Topology& t = topo_of(m);
    if (edges) std::memcpy(edges, t.edges.data(), sizeof(int) * t.edges.size());
    if (rest_len) std::memcpy(rest_len, t.rest_len.data(), sizeof(float) * t.rest_len.size());
    if (vt_ptr) std::memcpy(vt_ptr, t.vt_ptr.data(), sizeof(int) * t.vt_ptr.size());
    if (vt) std::memcpy(vt, t.vt.data(), sizeof(int) * t.vt.size());
    if (tri_tri) std::memcpy(tri_tri, t.tri_tri.data(), sizeof(int) * t.tri_tri.size());
    return PDG_OK;
    GUARD_END
}

// ----------------------------------------------------------- constraints
int pdg_constraints_create(const pdg_mesh* m, pdg_constraints** out)
{
    GUARD_BEGIN
    if (!m || !out) return set_error(PDG_ERR_ARG, "pdg_constraints_create: bad arguments");
    topo_of(m);
    pdg_constraints* c = new pdg_constraints;
    c->mesh = m->data;
    c->topo = m->topo;
    *out = c;
    return PDG_OK;
    GUARD_END
}

int pdg_constraints_build_stretch(pdg_constraints* c, float k)
{
    GUARD_BEGIN
    if (!c || !(k >= 0.f) || !std::isfinite(k)) return set_error(PDG_ERR_ARG, "pdg_constraints_build_stretch: bad stiffness");
    c->c.k_stretch.assign(c->mesh->T, k);
    return PDG_OK;
    GUARD_END
}

int pdg_constraints_set_stretch_k(pdg_constraints* c, const float* k)
{
    GUARD_BEGIN
    if (!c || !k) return set_error(PDG_ERR_ARG, "pdg_constraints_set_stretch_k: bad arguments");
    for (int t = 0; t < c->mesh->T; ++t)
        if (!(k[t] >= 0.f) || !std::isfinite(k[t])) return set_error(PDG_ERR_ARG, "stretch stiffness must be finite and >= 0");
    c->c.k_stretch.assign(k, k + c->mesh->T);
    return PDG_OK;
    GUARD_END
}

int pdg_constraints_build_bend(pdg_constraints* c, float k)
{
    GUARD_BEGIN
    if (!c || !(k >= 0.f) || !std::isfinite(k)) return set_error(PDG_ERR_ARG, "pdg_constraints_build_bend: bad stiffness");
    build_bend(*c->mesh, *c->topo, k, c->c);
    return PDG_OK;
    GUARD_END
}

int pdg_constraints_set_pins(pdg_constraints* c, const int* idx, int P, const float* targets)
{
    GUARD_BEGIN
    if (!c || P < 0 || (P > 0 && !idx)) return set_error(PDG_ERR_ARG, "pdg_constraints_set_pins: bad arguments");
    const MeshData& m = *c->mesh;
    std::vector<char> seen(m.N, 0);
    for (int q = 0; q < P; ++q) {
        if (idx[q] < 0 || idx[q] >= m.N) return set_error(PDG_ERR_ARG, "pin index %d out of range [0, %d)", idx[q], m.N);
        if (seen[idx[q]]) return set_error(PDG_ERR_ARG, "pin index %d listed twice", idx[q]);
        seen[idx[q]] = 1;
    }
    c->c.pins.assign(idx, idx + P);
    c->c.targets.resize(3 * (size_t)P);
    for (int q = 0; q < P; ++q)
        for (int d = 0; d < 3; ++d)
            c->c.targets[3 * q + d] = targets ? targets[3 * q + d] : m.rest[3 * idx[q] + d];
    return PDG_OK;
    GUARD_END
}

int pdg_constraints_pin_top_row(pdg_constraints* c, int ncols)
{
    GUARD_BEGIN
    if (!c || ncols < 1 || ncols > c->mesh->N) return set_error(PDG_ERR_ARG, "pin_top_row: ncols out of range");
    std::vector<int> idx(ncols);
    for (int j = 0; j < ncols; ++j) idx[j] = j;
    return pdg_constraints_set_pins(c, idx.data(), ncols, nullptr);
    GUARD_END
}

int pdg_constraints_pin_corners(pdg_constraints* c, int ncols)
{
    if (!c || ncols < 2 || ncols > c->mesh->N) return set_error(PDG_ERR_ARG, "pin_corners: ncols out of range");
    const int idx[2] = {0, ncols - 1};
    return pdg_constraints_set_pins(c, idx, 2, nullptr);
}

int pdg_constraints_counts(const pdg_constraints* c, int* nb, int* np)
{
    if (!c) return set_error(PDG_ERR_ARG, "null constraints");
    if (nb) *nb = (int)c->c.bend_k.size();
    if (np) *np = (int)c->c.pins.size();
    return PDG_OK;
}

int pdg_constraints_get(const pdg_constraints* c, float* k, int* quads, float* w, float* n_rest, float* bend_k,
                        int* pins, float* targets)
{
    if (!c) return set_error(PDG_ERR_ARG, "null constraints");
    const ConstraintData& d = c->c;
    if (k) std::memcpy(k, d.k_stretch.data(), sizeof(float) * d.k_stretch.size());
    if (quads) std::memcpy(quads, d.quads.data(), sizeof(int) * d.quads.size());
    if (w) std::memcpy(w, d.w.data(), sizeof(float) * d.w.size());
    if (n_rest) std::memcpy(n_rest, d.n_rest.data(), sizeof(float) * d.n_rest.size());
    if (bend_k) std::memcpy(bend_k, d.bend_k.data(), sizeof(float) * d.bend_k.size());
    if (pins) std::memcpy(pins, d.pins.data(), sizeof(int) * d.pins.size());
    if (targets) std::memcpy(targets, d.targets.data(), sizeof(float) * d.targets.size());
    return PDG_OK;
}

int pdg_constraints_jacobi_diag(const pdg_constraints* c, float dt, float* diag)
{
    GUARD_BEGIN
    if (!c || !diag || !(dt > 0.f)) return set_error(PDG_ERR_ARG, "pdg_constraints_jacobi_diag: bad arguments");
    std::vector<float> d;
    jacobi_diag(*c->mesh, c->c, dt, d);
    std::memcpy(diag, d.data(), sizeof(float) * d.size());
    return PDG_OK;
    GUARD_END
}

void pdg_constraints_destroy(pdg_constraints* c) { delete c; }

}  // extern "C"
