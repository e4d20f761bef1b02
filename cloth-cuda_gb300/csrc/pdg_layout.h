// Device data layout of the PD solver, shared by the host patch builder
// (layout.cpp) and the kernels (pd_kernels.cu).
//
// The cloths of a solver are concatenated in one Morton-reordered vertex
// numbering.  Each cloth's vertices are cut into patches of up to
// `patch_verts` consecutive vertices; one CUDA block processes one patch.  A
// patch carries every triangle and bend hinge that touches one of its owned
// vertices, with vertex references rewritten as 16-bit local indices into
// the patch's vertex list (owned vertices first, then the halo).
#pragma once

#include <cstdint>
#include <vector_types.h>

namespace pdg {

struct PatchHdr {            // 80 B
    int cloth;               // cloth index
    int vbegin;              // first owned vertex (global, reordered)
    int nown;                // owned vertices
    int nlocal;              // owned + halo
    int halo_off;            // into halo[]
    int tri_off, ntri;       // into tri_rec[]
    int hinge_off, nhinge;   // into hinge_rec[]
    int csr_off;             // into csr_ptr[] (nown + 1 entries, relative to ent_off)
    int ent_off;             // into csr_ent[]
    int nslot;               // 3*ntri + 4*nhinge contribution slots
    int nent;                // gather-list entries of the owned vertices
    int nbnd;                // owned vertices 0..nbnd-1 are in other patches' halos
    int ntri_a, nhin_a;      // records 0..ntri_a-1 / 0..nhin_a-1 touch one of them
    int vm_npad;             // vertex-major slots: contribution j of owned vertex l at j*vm_npad + l
    int vm_nslot;            // vertex-major slot array length
    int pad[2];
};

struct TriRec {              // 32 B
    float4   G;              // Dm_inv col-major (g00, g10, g01, g11)
    float    h2wA;           // h^2 * k_stretch * rest area
    uint32_t l01;            // local indices of corners 0 | 1 << 16
    uint32_t l2;             // local index of corner 2 | vertex-major slot of corner 0 << 16
    uint32_t vm12;           // vertex-major slots of corners 1 | 2 << 16 (0xffff: halo corner)
};

struct HingeRec {            // 32 B
    float4   w;              // cotangent weights w0..w3
    float    h2k;            // h^2 * bend stiffness
    float    nrest;          // rest curvature norm
    uint32_t l01;            // local indices v0 | v1 << 16
    uint32_t l23;            // local indices v2 | v3 << 16
};

// Static per-cloth parameters.
struct ClothInfo {
    int   vbegin, nverts;
    int   patch_begin, patch_end;
    int   max_iter;
    int   use_cheb, cheb_delay;
    int   mode;              // PDG_MODE_*
    int   init;              // PDG_INIT_*
    float h, damping, gamma, tol, rho;
    float ext[3];            // gravity (y) + wind
    int   pad;
};

// Per-cloth runtime state of the current frame.
struct ClothRT {
    int    active;           // still iterating
    int    used;             // iterate kept (x^used)
    int    status;           // PDG_OK / PDG_ERR_NUMERIC
    int    warm;             // learned start kept
    double res_y2;           // ||r(y_pinned)||^2
    double res0_2;           // ||r(x^0)||^2
    double resf_2;           // ||r(x^used)||^2, -1 if not evaluated
};

// Arguments of one fused sweep.
struct IterArgs {
    const PatchHdr*  patches;
    const int*       halo;
    const TriRec*    tris;
    const HingeRec*  hinges;
    const uint2*     hvm;         // per hinge: vertex-major slots of corners 0 | 1 << 16, 2 | 3 << 16
    const int*       csr_ptr;
    const uint16_t*  csr_ent;
    const ClothInfo* cinfo;
    ClothRT*         crt;
    const float*     omega;       // per cloth, omega_stride entries: omega_k
    int              omega_stride;
    const float4*    Y;           // inertial prediction, w = mass
    float4*          buf[2];      // iterate ping-pong, w = inv_diag (>= 0) or -1 (pinned)
    double*          acc;         // ||r(x^k)||^2 per cloth and sweep k
    int              acc_stride;  // sweeps + 1
    int              ncloth;
    int              have_final;  // evaluate r(x^max_iter) in an extra sweep
    int              warm_active; // learned start evaluated this frame (res_y2 set by the selection)
};

}  // namespace pdg
