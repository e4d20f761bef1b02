// Device data layout of the PD solver, shared by the host patch builder
// (layout.cpp) and the kernels (pd_kernels.cu).
//
// The cloths of a solver are concatenated in one reordered vertex numbering:
// recursive coordinate bisection of each cloth's rest shape into compact
// tiles of `patch_verts` vertices, Z-order inside a tile.  Each cloth's
// vertices are cut into patches of up to `patch_verts` consecutive vertices
// (one tile each); one CUDA block processes one patch.  A
// patch carries every cell and every lone bend hinge that touches one of its
// owned vertices, with vertex references rewritten as 16-bit local indices
// into the patch's vertex list (owned vertices first, then the halo).
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
    int cell_off, ncell;     // into cells[]
    int hinge_off, nhinge;   // into hinges[] (lone hinges)
    int csr_off;             // into csr_ptr[] (nown + 1 entries, relative to ent_off)
    int ent_off;             // into csr_ent[]
    int nslot;               // 6*ncell + 4*nhinge contribution slots
    int nent;                // gather-list entries of the owned vertices
    int nbnd;                // owned vertices 0..nbnd-1 are in other patches' halos
    int ncell_a, nhin_a;     // records 0..ncell_a-1 / 0..nhin_a-1 touch one of them
    int vm_npad;             // vertex-major slots: contribution j of owned vertex l at j*vm_npad + l
    int vm_nslot;            // vertex-major slot array length
    int pad[2];
};

// A cell groups the records around one pair of triangles so that their four
// shared corners are read once and their contributions are summed before
// they are stored:
//   t0 = (c0, c1, c2) and t1 = (c1, c0, c3), two triangles sharing the edge
//      c0-c1, corners rotated so that edge comes first (G in that order);
//   h0, the bend hinge of c0-c1, weights W0 over c0..c3;
//   h1, h2, up to two hinges of the pair's outer edges, each with three
//      corners among c0..c3 (weights W1, W2) and one outer corner x1 / x2
//      (weight wx1 / wx2).
// Absent parts carry zero weights and stiffness: a lone triangle has G1 = 0
// and c3 = c0.  Outputs o0..o3 are the summed contributions to c0..c3 and
// o4 / o5 those to x1 / x2.
// On the device the records of a patch are stored in groups of kCellGroup:
// 16-byte piece i of record c of a patch at piece index
// cell_off * 9 + (c / 8) * 72 + i * 8 + c % 8, so that a warp's load of piece
// i of 32 consecutive records reads four whole 128-byte lines (on the host,
// L.cells holds them record after record).  Every patch's records start on a
// multiple of kCellGroup; the layout pads the gaps with unused records.
constexpr int kCellGroup = 8;

struct CellRec {             // 144 B
    float4   G0, G1;         // Dm_inv of t0, t1, col-major (g00, g10, g01, g11)
    float4   W0, W1, W2;     // weights of c0..c3 in h0, h1, h2
    float    h2wA0, h2wA1;   // h^2 * k_stretch * rest area of t0, t1
    float    h2k0, nrest0;   // h0: h^2 * bend stiffness, rest curvature norm
    float    h2k1, nrest1, wx1;
    float    h2k2, nrest2, wx2;
    uint32_t c01, c23;       // local indices c0 | c1 << 16, c2 | c3 << 16
    uint32_t x12;            // local indices x1 | x2 << 16 (c0 when absent)
    uint32_t vm01, vm23, vm45;   // vertex-major slots of o0..o5 (0xffff: halo corner or absent)
};

// A bend hinge that no cell holds.
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
    const CellRec*   cells;
    const HingeRec*  hinges;
    const uint2*     hvm;         // per hinge: vertex-major slots of corners 0 | 1 << 16, 2 | 3 << 16
    const int*       csr_ptr;
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
