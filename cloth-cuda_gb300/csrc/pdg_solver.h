// Internal solver object of the PD cloth library.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include "../../include/pdg.h"
#include "pdg_host.h"
#include "pdg_kernels.h"
#include "pdg_layout.h"

namespace pdg {

struct ClothSetup {
    std::shared_ptr<const MeshData> mesh;
    std::shared_ptr<const Topology> topo;
    ConstraintData cons;
    pdg_config cfg;
};

struct HostLayout {
    int ntot = 0, ncloth = 0, npatch = 0, cap = 0, omega_stride = 1;
    int max_nlocal = 0, max_nslot = 0, max_nown = 0, max_ncell = 0, max_nhinge = 0, max_nent = 0, max_nhalo = 0;
    size_t smem_bytes = 0;          // per-patch sweep kernels (vertex-major slots)
    size_t max_vm_slot = 0;         // largest 32*nlocal + 12*vm_nslot of a patch
    int max_vm_nslot = 0;           // largest vertex-major slot count of a patch
    size_t smem_resident = 0;       // resident kernel: records, y, d, slots, gather lists
    std::vector<int> perm_global;   // reordered vertex -> index in the batch's caller order
    std::vector<int> perm_local;    // reordered vertex -> index within its cloth
    std::vector<int> vcloth;
    std::vector<float> mass;
    std::vector<float4> aux;
    std::vector<ClothInfo> cinfo;
    std::vector<float> omega;
    std::vector<PatchHdr> patches;
    std::vector<int> halo;
    std::vector<CellRec> cells;
    std::vector<HingeRec> hinges;
    std::vector<uint2> hvm;         // per hinge: its vertex-major slot addresses
    std::vector<int> csr_ptr;
    std::vector<uint16_t> csr_ent;
    std::vector<int> nbr_ptr, nbr;  // patches owning each patch's halo vertices
};

bool build_layout(const std::vector<ClothSetup>& cl, int patch_verts, HostLayout& L, std::string& err);
// The properties the sweep kernels rely on (partition, halo, neighbour lists,
// boundary-first order, each contribution slot written once, every incident
// triangle held): empty if they hold, else the first violation.
std::string check_layout(const std::vector<ClothSetup>& cl, const HostLayout& L);

// Owning device allocation.
template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { if (p) cudaFree(p); }
    cudaError_t alloc(size_t count)
    {
        if (p) { cudaFree(p); p = nullptr; }
        n = count;
        return cudaMalloc(&p, sizeof(T) * (count ? count : 1));
    }
    cudaError_t upload(const std::vector<T>& h, cudaStream_t s)
    {
        cudaError_t e = alloc(h.size());
        if (e != cudaSuccess || h.empty()) return e;
        return cudaMemcpyAsync(p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, s);
    }
};

}  // namespace pdg

struct pdg_solver {
    std::vector<pdg::ClothSetup> cloths;
    pdg::HostLayout L;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int kernel = PDG_KERNEL_GRAPH;
    int patch_verts = 256;
    int nt = 256;
    int mode = PDG_MODE_CONSISTENT;
    int have_final = 1;
    int persist_grid = 0;           // persistent / resident / streaming grid
    int res_variant = -1;           // resident kernel instance (record capacity)
    int carveout = 0;               // shared/L1 split of the per-sweep kernel (percent, 0 = default)
    pdg::StreamArgs sargs{};        // streaming kernel: stage layout
    size_t stream_smem = 0;
    long long launches = 0;
    long long wait_budget = 2000000000LL;   // clock64 cycles per bounded wait (~1 s)
    int kernels_per_frame = 0;

    pdg::DevBuf<float4> X, V, Y, A, B, aux, warm;
    // learned start (allocated when a network is attached): the previous
    // frame's offset per vertex (w = 1 valid), and the learned chain's
    // iterates, records and per-sweep sums for the judge after K sweeps
    pdg::DevBuf<float4> dprev, A2, B2;
    pdg::DevBuf<pdg::ClothRT> crt2;
    pdg::DevBuf<double> acc2;
    pdg::DevBuf<float> mass, omega, stage_x, stage_v;
    pdg::DevBuf<int> vcloth, perm_global, perm_local, halo, csr_ptr;
    pdg::DevBuf<int> inv_global;   // caller-order index in the batch -> reordered vertex
    pdg::DevBuf<double> acc;
    // resident kernel: tagged boundary offsets exchanged between patches
    // (2 x vertices x 4 words) and the device word holding the next frame's
    // tag base
    pdg::DevBuf<unsigned long long> xch;
    pdg::DevBuf<unsigned> xch_tag;
    int acc_stride = 1;
    int nbr_sync = 0;
    pdg::DevBuf<pdg::PatchHdr> patches;
    pdg::DevBuf<pdg::CellRec> cells;
    pdg::DevBuf<pdg::HingeRec> hinges;
    pdg::DevBuf<uint2> hvm;
    pdg::DevBuf<pdg::ClothInfo> cinfo;
    pdg::DevBuf<pdg::ClothRT> crt;
    pdg::DevBuf<unsigned> bar;

    cudaGraphExec_t graph = nullptr;
    std::vector<pdg::ClothRT> h_rt;
    bool warm_valid = false;
    pdg_warmstart* ws = nullptr;   // attached learned warm start (not owned)
    bool any_warm = false;         // some cloth asks for a learned start
    bool any_keep = false;         // some cloth always keeps it (PDG_INIT_WARMSTART_KEEP)
    std::vector<pdg_tune_entry> tune;   // autotuner candidate table

    ~pdg_solver();
};

namespace pdg {
// solver creation with a concrete launch plan (solver.cpp) and through the
// autotuner (tune.cpp)
int create_solver(int n, const pdg_config* cfgs, const pdg_mesh* const* meshes, const pdg_constraints* const* cons,
                  void* stream, pdg_solver** out);
int autotune_create(int n, const pdg_config* cfgs, const pdg_mesh* const* meshes, const pdg_constraints* const* cons,
                    void* stream, pdg_solver** out);
// learned warm start hooks (gnn.cu): features + forward into s->warm
int warm_infer_enqueue(pdg_warmstart* w, pdg_solver* s);
int warm_kernel_count();
// sweeps each start runs before the judge compares them (0: compare the
// start residuals)
int warm_judge_sweeps(const pdg_warmstart* w);
void warm_detach(pdg_warmstart* w);
}  // namespace pdg
