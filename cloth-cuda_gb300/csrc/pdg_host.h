// Internal host-side data of the PD cloth library (not part of the ABI).
#pragma once

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

namespace pdg {

// Immutable rest mesh + rest state (ClothMesh, include/cloth_mesh.h:18-67).
struct MeshData {
    int N = 0, T = 0;
    float density = 0.1f;
    std::vector<float> rest;     // N*3
    std::vector<int>   tris;     // T*3
    std::vector<float> Dm_inv;   // T*4 col-major (g00, g10, g01, g11)
    std::vector<float> area;     // T
    std::vector<float> mass;     // N
};

// MeshTopology (include/mesh_topology.h:12-30).
struct Topology {
    std::vector<int>   edges;     // E*4 (v0, v1, tri_a, tri_b), sorted by (v0, v1)
    std::vector<float> rest_len;  // E
    std::vector<int>   vt_ptr;    // N+1
    std::vector<int>   vt;        // 3T vertex->triangle lists
    std::vector<int>   tri_tri;   // T*3 neighbour opposite each corner
    int num_inner = 0;
};

// SimConstraints (include/sim_constraints.h:30-78) + Constraints pins.
struct ConstraintData {
    std::vector<float> k_stretch;   // T
    std::vector<int>   quads;       // E*4
    std::vector<float> w;           // E*4
    std::vector<float> n_rest;      // E
    std::vector<float> bend_k;      // E
    std::vector<int>   pins;        // P
    std::vector<float> targets;     // P*3
};

// ---- setup (setup.cpp) ----
void generate_grid(int nrows, int ncols, float size, int type,
                   std::vector<float>& pos, std::vector<int>& tris);
void precompute_rest_state(MeshData& m);
void build_topology(const MeshData& m, Topology& t);
void build_bend(const MeshData& m, const Topology& t, float k, ConstraintData& c);
void jacobi_diag(const MeshData& m, const ConstraintData& c, float dt, std::vector<float>& diag);
bool load_obj(const std::string& path, std::vector<float>& pos, std::vector<int>& tris,
              std::string& err);
uint64_t splitmix64(uint64_t& s);
double gaussian(uint64_t& s);

// ---- error reporting (capi.cpp) ----
int set_error(int code, const char* fmt, ...);

}  // namespace pdg

struct pdg_mesh {
    std::shared_ptr<const pdg::MeshData> data;
    std::shared_ptr<const pdg::Topology> topo;   // built on first use
};

struct pdg_constraints {
    std::shared_ptr<const pdg::MeshData> mesh;
    std::shared_ptr<const pdg::Topology> topo;
    pdg::ConstraintData c;
};
