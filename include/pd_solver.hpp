// pd_solver.hpp -- C++ shim with the reference's class shapes over the C ABI.
//
// Header-only.  Mirrors the interfaces a cloth-cuda driver uses
// (include/pd_solver.h, include/cloth_mesh.h, include/mesh_topology.h,
// include/sim_constraints.h, include/constraints.h, include/mesh_generator.h)
// so that a sim_cloth-style program ports by changing its includes and
// namespace.  Differences: the simulation state lives in the solver (on the
// GPU); read it back with PDSolver::download(mesh), which fills
// mesh.pos_cpu / vel_cpu, and write it with PDSolver::upload(mesh).  Errors
// throw cloth_pdg::Error instead of exiting the process.
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

#include "pdg.h"

namespace cloth_pdg {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& what) : std::runtime_error(what), code(c) {}
};

inline void check(int rc)
{
    if (rc != PDG_OK) throw Error(rc, pdg_last_error_string());
}

// include/pd_solver.h:4-15 (same fields and defaults)
struct PDSolverConfig {
    int   max_iterations = 50;
    float tolerance = 1e-4f;            // the reference never reads it; see use_tolerance
    bool  use_chebyshev = true;
    bool  use_cpu_stretch_reference = false;   // not supported: there is no CPU path
    float rho = 0.9f;
    float gravity = -9.8f;
    float dt = 0.01f;
    float stretch_stiffness = 1.0f;
    float bend_stiffness = 0.0f;
    float damping = 0.0f;
    // extensions
    bool  use_tolerance = false;        // stop at `tolerance` relative residual
    bool  reference_literal = false;    // reproduce src/pd_solver.cu's update
};

// include/cloth_mesh.h:18-67 (geometry + rest state; GPU buffers live in the solver)
struct ClothMesh {
    pdg_mesh* h = nullptr;
    int num_verts = 0, num_tris = 0;
    std::vector<float> rest_pos;    // N*3
    std::vector<int> triangles;     // T*3
    std::vector<float> pos_cpu, vel_cpu;   // filled by PDSolver::download

    ClothMesh() = default;
    ClothMesh(const ClothMesh&) = delete;
    ClothMesh& operator=(const ClothMesh&) = delete;
    ~ClothMesh() { if (h) pdg_mesh_destroy(h); }

    void adopt(pdg_mesh* m)
    {
        if (h) pdg_mesh_destroy(h);
        h = m;
        check(pdg_mesh_counts(h, &num_verts, &num_tris));
        rest_pos.resize(3 * (size_t)num_verts);
        triangles.resize(3 * (size_t)num_tris);
        check(pdg_mesh_get(h, rest_pos.data(), triangles.data(), nullptr, nullptr, nullptr, nullptr));
        pos_cpu = rest_pos;
        vel_cpu.assign(rest_pos.size(), 0.f);
    }
    // ClothMesh::load_obj (src/cloth_mesh.cpp:89-132); density as precompute_rest_state
    bool load_obj(const std::string& path, float density = 0.1f)
    {
        pdg_mesh* m = nullptr;
        if (pdg_mesh_load_obj(path.c_str(), density, &m) != PDG_OK) return false;
        adopt(m);
        return true;
    }
    // rest state for caller-filled rest_pos / triangles
    void precompute_rest_state(float density = 0.1f)
    {
        pdg_mesh* m = nullptr;
        check(pdg_mesh_create(rest_pos.data(), (int)(rest_pos.size() / 3), triangles.data(),
                              (int)(triangles.size() / 3), density, &m));
        adopt(m);
    }
    std::vector<float> mass() const
    {
        std::vector<float> m(num_verts);
        check(pdg_mesh_get(h, nullptr, nullptr, nullptr, nullptr, m.data(), nullptr));
        return m;
    }
};

// include/mesh_generator.h:14 (x-z plane, `size` = cell edge), rest state at density 0.1
inline void generate_square_cloth(int nrows, int ncols, float size, int type, ClothMesh& mesh,
                                  float density = 0.1f)
{
    pdg_mesh* m = nullptr;
    check(pdg_mesh_generate(nrows, ncols, size, type, density, &m));
    mesh.adopt(m);
}

// include/mesh_topology.h:12-30
struct MeshTopology {
    struct EdgeTopo { int v0, v1, tri_a, tri_b; float rest_len; };
    std::vector<EdgeTopo> edges;
    int inner = 0;
    int num_inner_edges() const { return inner; }
    static MeshTopology build(const ClothMesh& mesh)
    {
        MeshTopology t;
        int ne = 0;
        check(pdg_topology_counts(mesh.h, &ne, &t.inner));
        std::vector<int> e(4 * (size_t)ne);
        std::vector<float> len(ne);
        check(pdg_topology_get(mesh.h, e.data(), len.data(), nullptr, nullptr, nullptr));
        for (int i = 0; i < ne; ++i) t.edges.push_back({e[4 * i], e[4 * i + 1], e[4 * i + 2], e[4 * i + 3], len[i]});
        return t;
    }
};

// include/sim_constraints.h:30-78
struct SimConstraints {
    pdg_constraints* h = nullptr;
    int num_tris = 0, num_bend_cons = 0;
    SimConstraints() = default;
    SimConstraints(const SimConstraints&) = delete;
    SimConstraints& operator=(const SimConstraints&) = delete;
    ~SimConstraints() { if (h) pdg_constraints_destroy(h); }
    void ensure(const ClothMesh& mesh)
    {
        if (!h) check(pdg_constraints_create(mesh.h, &h));
        num_tris = mesh.num_tris;
    }
    void build_stretch(const ClothMesh& mesh, float stiffness)
    {
        ensure(mesh);
        check(pdg_constraints_build_stretch(h, stiffness));
    }
    void build_bend(const ClothMesh& mesh, const MeshTopology&, float stiffness)
    {
        ensure(mesh);
        check(pdg_constraints_build_bend(h, stiffness));
        int np = 0;
        check(pdg_constraints_counts(h, &num_bend_cons, &np));
    }
    // the solver computes the diagonal for its dt; kept for source compatibility
    void precompute_jacobi_diag(const ClothMesh&, float) {}
    void upload_to_gpu() {}
};

// include/constraints.h:5-36
struct Constraints {
    std::vector<int> pinned_indices;
    std::vector<float> target_positions;   // num_verts * 3, as in the reference
    void set_from_list(const std::vector<int>& indices, const ClothMesh& mesh)
    {
        pinned_indices = indices;
        target_positions.assign(3 * (size_t)mesh.num_verts, 0.f);
        for (int i : indices)
            for (int d = 0; d < 3; ++d) target_positions[3 * i + d] = mesh.rest_pos[3 * i + d];
    }
    void pin_top_row(const ClothMesh& mesh, int ncols)
    {
        std::vector<int> idx(ncols);
        for (int j = 0; j < ncols; ++j) idx[j] = j;
        set_from_list(idx, mesh);
    }
    void pin_corners(const ClothMesh& mesh, int ncols) { set_from_list({0, ncols - 1}, mesh); }
    void clear() { pinned_indices.clear(); target_positions.clear(); }
    void upload_to_gpu() {}
};

// include/pd_solver.h:30-71
class PDSolver {
public:
    PDSolver(const PDSolverConfig& cfg, const ClothMesh& mesh, const SimConstraints&) : cfg_(cfg), n_(mesh.num_verts)
    {
        if (cfg.use_cpu_stretch_reference)
            throw Error(PDG_ERR_ARG, "the CPU stretch reference is not part of this library");
    }
    PDSolver(const PDSolver&) = delete;
    PDSolver& operator=(const PDSolver&) = delete;
    ~PDSolver() { if (s_) pdg_solver_destroy(s_); }

    // PDSolver::step (src/pd_solver.cu:496-621).  The first call builds the
    // GPU solver (the cloth starts at rest); later calls pass a changed pin
    // list or changed pin targets on to it, as the reference's
    // Constraints::upload_to_gpu re-uploads them (src/constraints.cpp:77-101).
    void step(ClothMesh& mesh, SimConstraints& sim, const Constraints& pins)
    {
        if (!s_) {
            build(mesh, sim, pins);
        } else {
            std::vector<float> tgt = targets_of(pins);
            if (pins.pinned_indices != pins_)
                check(pdg_solver_set_pins(s_, 0, pins.pinned_indices.data(), (int)pins.pinned_indices.size(),
                                          tgt.empty() ? nullptr : tgt.data()));
            else if (tgt != tgt_ && !tgt.empty())
                check(pdg_solver_set_pin_targets(s_, 0, tgt.data()));
            pins_ = pins.pinned_indices;
            tgt_ = tgt;
        }
        check(pdg_solver_step(s_, 1, &last_));
    }
    void reset() { if (s_) check(pdg_solver_reset(s_)); }
    void download(ClothMesh& mesh)
    {
        mesh.pos_cpu.resize(3 * (size_t)n_);
        mesh.vel_cpu.resize(3 * (size_t)n_);
        check(pdg_solver_get_state(s_, 0, mesh.pos_cpu.data(), mesh.vel_cpu.data(), 0));
    }
    void upload(const ClothMesh& mesh) { check(pdg_solver_set_state(s_, 0, mesh.pos_cpu.data(), mesh.vel_cpu.data(), 0)); }
    const pdg_frame_stats& last_stats() const { return last_; }

private:
    static std::vector<float> targets_of(const Constraints& pins)
    {
        std::vector<float> tgt;
        for (int i : pins.pinned_indices)
            for (int d = 0; d < 3; ++d) tgt.push_back(pins.target_positions[3 * i + d]);
        return tgt;
    }
    void build(ClothMesh& mesh, SimConstraints& sim, const Constraints& pins)
    {
        sim.ensure(mesh);
        const std::vector<float> tgt = targets_of(pins);
        check(pdg_constraints_set_pins(sim.h, pins.pinned_indices.data(), (int)pins.pinned_indices.size(),
                                       tgt.empty() ? nullptr : tgt.data()));
        pdg_config c;
        check(pdg_config_default(&c));
        c.max_iterations = cfg_.max_iterations;
        c.tolerance = cfg_.use_tolerance ? cfg_.tolerance : 0.f;
        c.use_chebyshev = cfg_.use_chebyshev;
        c.rho = cfg_.rho;
        c.gravity = cfg_.gravity;
        c.dt = cfg_.dt;
        c.stretch_stiffness = cfg_.stretch_stiffness;
        c.bend_stiffness = cfg_.bend_stiffness;
        c.damping = cfg_.damping;
        if (cfg_.reference_literal) { c.mode = PDG_MODE_REFERENCE_LITERAL; c.init = PDG_INIT_PREVIOUS; }
        check(pdg_solver_create(&c, mesh.h, sim.h, nullptr, &s_));
        pins_ = pins.pinned_indices;
        tgt_ = tgt;
    }
    PDSolverConfig cfg_;
    int n_;
    pdg_solver* s_ = nullptr;
    std::vector<int> pins_;
    std::vector<float> tgt_;
    pdg_frame_stats last_{};
};

}  // namespace cloth_pdg
