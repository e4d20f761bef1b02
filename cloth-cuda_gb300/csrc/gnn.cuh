// Learned warm start: shapes, parameter layout and device kernels of the
// mesh message-passing network (no counterpart in the reference).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cstdint>

namespace pdg {
namespace gnn {

constexpr int H = 64;      // hidden width
constexpr int NF = 14;     // node features
constexpr int NFP = 16;    // node features padded to one mma k-step
constexpr int EF = 4;      // edge features
constexpr int NO = 3;      // outputs
constexpr int NOP = 8;     // outputs padded to one mma n-tile
constexpr int L = 2;       // message-passing layers
// length scales of the features: offsets and velocities in units of one
// frame's gravity drop h^2 g at h = 1/60; rest lengths relative to 1 cm.
// Node features: (y - x_n)/s, h v_n/s, pinned flag, log mass, log stretch k,
// log bend k, the previous frame's offset d_prev/s and its validity flag.
constexpr float kOffsetScale = 2.725e-3f;
constexpr float kLenScale = 0.01f;

// Flat fp32 parameter vector, in this order (the order of pdg_warmstart_get_params):
// We[H][NF] be[H] {A[H][H] B[H][H] C[H][EF] c[H] U[H][2H] u[H]} x L  Wd[NO][H] bd[NO]
struct Layout {
    int We, be, A[L], B[L], C[L], c[L], U[L], u[L], Wd, bd, total;
    Layout()
    {
        int o = 0;
        We = o; o += H * NF;
        be = o; o += H;
        for (int l = 0; l < L; ++l) {
            A[l] = o; o += H * H;
            B[l] = o; o += H * H;
            C[l] = o; o += H * EF;
            c[l] = o; o += H;
            U[l] = o; o += H * 2 * H;
            u[l] = o; o += H;
        }
        Wd = o; o += NO * H;
        bd = o; o += NO;
        total = o;
    }
};

// bf16 copies of the weights laid out for the GEMM kernel (W[nout][k]) and
// their transposes for the data gradients.
struct Bf16Weights {
    __nv_bfloat16* We;        // [H][NFP]
    __nv_bfloat16* AB[L];     // [2H][H]  rows 0..H-1 = A, H..2H-1 = B
    __nv_bfloat16* ABt[L];    // [H][2H]
    __nv_bfloat16* U[L];      // [H][2H]
    __nv_bfloat16* Ut[L];     // [2H][H]
    __nv_bfloat16* Wd;        // [NOP][H] (rows >= NO zero)
    __nv_bfloat16* Wdt;       // [H][NOP]
};

}  // namespace gnn
}  // namespace pdg
