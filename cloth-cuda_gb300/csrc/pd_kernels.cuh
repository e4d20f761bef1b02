// Device-side pieces of the PD solve shared by the per-sweep kernel, the
// persistent kernel and the resident kernel.  All arithmetic on the solve
// path uses explicitly rounded intrinsics, so the three launch structures
// give bitwise identical results whatever the surrounding code.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "pdg_layout.h"

namespace pdg {

enum { kModeConsistent = 0, kModeLiteral = 1 };

__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float ffma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return ffma(a.x, b.x, ffma(a.y, b.y, fmul(a.z, b.z))); }
__device__ __forceinline__ float3 scale3(float3 a, float s) { return make_float3(fmul(a.x, s), fmul(a.y, s), fmul(a.z, s)); }
__device__ __forceinline__ float3 f3(float4 a) { return make_float3(a.x, a.y, a.z); }
__device__ __forceinline__ float3 fadd3(float3 a, float3 b)
{
    return make_float3(fadd(a.x, b.x), fadd(a.y, b.y), fadd(a.z, b.z));
}

// ---------------------------------------------------------------------------
// Stretch projection, consistent form: Gram-Schmidt basis (b0, b1) of F's
// columns, F2d = [b0 b1]^T F, closest rotation in SO(2) in closed form
// R2d = rot(atan2(F2d10 - F2d01, F2d00 + F2d11)) with (cos, sin) formed by
// normalising (F2d00 + F2d11, F2d10 - F2d01), R = [b0 b1] R2d.  This is
// the projection of src/stretch_reference.cpp:38-68 (JacobiSVD U V^T with the
// determinant fix) without the SVD.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void polar_consistent(float3 F0, float3 F1, float3& R0, float3& R1)
{
    const float n0sq = dot3(F0, F0);
    const float3 b0 = n0sq > 1e-20f ? scale3(F0, rsqrtf(n0sq)) : make_float3(1.f, 0.f, 0.f);
    const float a01 = dot3(F1, b0);
    const float3 c1 = make_float3(ffma(-a01, b0.x, F1.x), ffma(-a01, b0.y, F1.y), ffma(-a01, b0.z, F1.z));
    const float n1sq = dot3(c1, c1);
    float3 b1;
    if (n1sq > 1e-20f) {
        b1 = scale3(c1, rsqrtf(n1sq));
    } else {   // F1 parallel to F0: any unit vector orthogonal to b0
        float3 q = make_float3(-b0.y, b0.x, 0.f);
        float nq = ffma(q.x, q.x, fmul(q.y, q.y));
        if (nq < 1e-20f) { q = make_float3(0.f, -b0.z, b0.y); nq = ffma(q.y, q.y, fmul(q.z, q.z)); }
        b1 = scale3(q, rsqrtf(nq));
    }
    const float a00 = dot3(b0, F0), a10 = dot3(b1, F0), a11 = dot3(b1, F1);
    const float s = fadd(a00, a11), t = fsub(a10, a01);
    const float rr = ffma(s, s, fmul(t, t));
    float c = 1.f, sn = 0.f;
    if (rr > 1e-30f) { const float r = rsqrtf(rr); c = fmul(s, r); sn = fmul(t, r); }
    R0 = make_float3(ffma(b0.x, c, fmul(b1.x, sn)), ffma(b0.y, c, fmul(b1.y, sn)), ffma(b0.z, c, fmul(b1.z, sn)));
    R1 = make_float3(ffma(b1.x, c, fmul(-b0.x, sn)), ffma(b1.y, c, fmul(-b0.y, sn)), ffma(b1.z, c, fmul(-b0.z, sn)));
}

// ---------------------------------------------------------------------------
// Stretch projection with the semantics of the reference kernel
// tri_stretch_project_kernel (src/pd_solver.cu:48-208): eigenvectors V of
// F2d^T F2d, W = F2d V / sigma, R2d = V W^T (the transpose of the polar
// rotation), R = U R2d.  Used only by the reference-literal mode.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void polar_literal(float3 F0, float3 F1, float3& R0, float3& R1)
{
    const float lf0 = __fsqrt_rn(dot3(F0, F0));
    const float3 u1 = lf0 > 1e-10f ? make_float3(fdiv(F0.x, lf0), fdiv(F0.y, lf0), fdiv(F0.z, lf0))
                                   : make_float3(1.f, 0.f, 0.f);
    const float f1u1 = dot3(F1, u1);
    const float3 up = make_float3(fsub(F1.x, fmul(f1u1, u1.x)), fsub(F1.y, fmul(f1u1, u1.y)),
                                  fsub(F1.z, fmul(f1u1, u1.z)));
    const float lup = __fsqrt_rn(dot3(up, up));
    float3 u2;
    if (lup > 1e-10f) {
        u2 = make_float3(fdiv(up.x, lup), fdiv(up.y, lup), fdiv(up.z, lup));
    } else {
        u2 = fabsf(u1.x) > 0.9f ? make_float3(-u1.y, u1.x, 0.f) : make_float3(0.f, -u1.z, u1.y);
        const float l = __fsqrt_rn(dot3(u2, u2));
        u2 = make_float3(fdiv(u2.x, l), fdiv(u2.y, l), fdiv(u2.z, l));
    }
    const float F00 = dot3(u1, F0), F01 = dot3(u1, F1), F10 = dot3(u2, F0), F11 = dot3(u2, F1);
    const float A00 = ffma(F00, F00, fmul(F10, F10));
    const float A01 = ffma(F00, F01, fmul(F10, F11));
    const float A11 = ffma(F01, F01, fmul(F11, F11));
    const float tr = fmul(fadd(A00, A11), 0.5f);
    const float dd = fsub(A00, A11);
    const float disc = __fsqrt_rn(fmaxf(0.f, ffma(fmul(dd, dd), 0.25f, fmul(A01, A01))));
    const float l1 = fadd(tr, disc), l2 = fsub(tr, disc);
    float v1x = 1.f, v1y = 0.f, v2x = 0.f, v2y = 1.f;
    if (!(disc < 1e-10f || fabsf(A01) < 1e-10f)) {
        const float tmp = fsub(l1, A00);
        const float l = __fsqrt_rn(ffma(A01, A01, fmul(tmp, tmp)));
        if (l > 1e-10f) { v1x = fdiv(A01, l); v1y = fdiv(tmp, l); }
        v2x = -v1y; v2y = v1x;
    }
    const float s1 = __fsqrt_rn(fmaxf(0.f, l1)), s2 = __fsqrt_rn(fmaxf(0.f, l2));
    float w1x = 1.f, w1y = 0.f, w2x, w2y;
    if (s1 > 1e-10f) {
        w1x = fdiv(ffma(F00, v1x, fmul(F01, v1y)), s1);
        w1y = fdiv(ffma(F10, v1x, fmul(F11, v1y)), s1);
    }
    if (s2 > 1e-10f) {
        w2x = fdiv(ffma(F00, v2x, fmul(F01, v2y)), s2);
        w2y = fdiv(ffma(F10, v2x, fmul(F11, v2y)), s2);
    } else {
        const float fx = ffma(F00, v2x, fmul(F01, v2y)), fy = ffma(F10, v2x, fmul(F11, v2y));
        const float d = ffma(w1x, fx, fmul(w1y, fy));
        const float wx = fsub(fx, fmul(d, w1x)), wy = fsub(fy, fmul(d, w1y));
        const float l = __fsqrt_rn(ffma(wx, wx, fmul(wy, wy)));
        if (l > 1e-10f) { w2x = fdiv(wx, l); w2y = fdiv(wy, l); } else { w2x = -w1y; w2y = w1x; }
    }
    const float r00 = ffma(v1x, w1x, fmul(v2x, w2x)), r01 = ffma(v1x, w1y, fmul(v2x, w2y));
    const float r10 = ffma(v1y, w1x, fmul(v2y, w2x)), r11 = ffma(v1y, w1y, fmul(v2y, w2y));
    R0 = make_float3(ffma(u1.x, r00, fmul(u2.x, r10)), ffma(u1.y, r00, fmul(u2.y, r10)), ffma(u1.z, r00, fmul(u2.z, r10)));
    R1 = make_float3(ffma(u1.x, r01, fmul(u2.x, r11)), ffma(u1.y, r01, fmul(u2.y, r11)), ffma(u1.z, r01, fmul(u2.z, r11)));
}

// Positions are carried as x = y + d: y the inertial prediction, d the
// offset the solve iterates on.  Edge vectors are formed as
// (y_j - y_i) + (d_j - d_i), so their rounding error is that of the small
// offsets, not of coordinates of size ~1 m.
__device__ __forceinline__ float3 edge(const float4* sy, const float4* sd, int i, int j)
{
    const float4 yi = sy[i], yj = sy[j], di = sd[i], dj = sd[j];
    return make_float3(fadd(fsub(yj.x, yi.x), fsub(dj.x, di.x)), fadd(fsub(yj.y, yi.y), fsub(dj.y, di.y)),
                       fadd(fsub(yj.z, yi.z), fsub(dj.z, di.z)));
}

// Corner contributions of one triangle from its two edge vectors:
// c_v = h^2 wA sum_col coef_{v,col} (R - F)_col (consistent) or with R alone
// (literal), coef from Dm_inv G = (g00, g10, g01, g11).
template <int MODE>
__device__ __forceinline__ void tri_force(float3 d1, float3 d2, float4 G, float h2wA, float3& c0, float3& c1,
                                          float3& c2)
{
    const float g00 = G.x, g10 = G.y, g01 = G.z, g11 = G.w;
    const float3 F0 = make_float3(ffma(d1.x, g00, fmul(d2.x, g10)), ffma(d1.y, g00, fmul(d2.y, g10)),
                                  ffma(d1.z, g00, fmul(d2.z, g10)));
    const float3 F1 = make_float3(ffma(d1.x, g01, fmul(d2.x, g11)), ffma(d1.y, g01, fmul(d2.y, g11)),
                                  ffma(d1.z, g01, fmul(d2.z, g11)));
    float3 R0, R1, q0, q1;
    if (MODE == kModeConsistent) {
        polar_consistent(F0, F1, R0, R1);
        q0 = make_float3(fmul(h2wA, fsub(R0.x, F0.x)), fmul(h2wA, fsub(R0.y, F0.y)), fmul(h2wA, fsub(R0.z, F0.z)));
        q1 = make_float3(fmul(h2wA, fsub(R1.x, F1.x)), fmul(h2wA, fsub(R1.y, F1.y)), fmul(h2wA, fsub(R1.z, F1.z)));
    } else {
        polar_literal(F0, F1, R0, R1);
        q0 = scale3(R0, h2wA);
        q1 = scale3(R1, h2wA);
    }
    const float s0 = -fadd(g00, g10), s1 = -fadd(g01, g11);
    c0 = make_float3(ffma(s0, q0.x, fmul(s1, q1.x)), ffma(s0, q0.y, fmul(s1, q1.y)), ffma(s0, q0.z, fmul(s1, q1.z)));
    c1 = make_float3(ffma(g00, q0.x, fmul(g01, q1.x)), ffma(g00, q0.y, fmul(g01, q1.y)), ffma(g00, q0.z, fmul(g01, q1.z)));
    c2 = make_float3(ffma(g10, q0.x, fmul(g11, q1.x)), ffma(g10, q0.y, fmul(g11, q1.y)), ffma(g10, q0.z, fmul(g11, q1.z)));
}

// Hinge: e = sum w_i x_i, target p = e * n_rest / |e| (0 if |e| or
// n_rest <= 1e-10, src/pd_solver.cu:304-335); corner i receives w_i q with
// q = h^2 k (p - e) (consistent) or h^2 k p (literal).  The consistent form
// scales by n_rest * rsqrt(|e|^2), like the stretch projection; the literal
// form keeps the reference kernel's square root and division.
template <int MODE>
__device__ __forceinline__ float3 hinge_q(float3 e, float h2k, float nrest)
{
    float3 p = make_float3(0.f, 0.f, 0.f);
    if (MODE == kModeConsistent) {
        const float n2 = dot3(e, e);
        if (nrest > 1e-10f && n2 > 1e-20f) p = scale3(e, fmul(nrest, rsqrtf(n2)));
        return make_float3(fmul(h2k, fsub(p.x, e.x)), fmul(h2k, fsub(p.y, e.y)), fmul(h2k, fsub(p.z, e.z)));
    }
    if (nrest > 1e-10f) {
        const float len = __fsqrt_rn(dot3(e, e));
        if (len > 1e-10f) p = scale3(e, fdiv(nrest, len));
    }
    return scale3(p, h2k);
}

// e = sum w_i x_i formed as sum_{i>0} w_i (x_i - x_0) + (sum w_i) x_0 from
// edge vectors.
template <int MODE>
__device__ __forceinline__ float3 hinge_force(float3 e1, float3 e2, float3 e3, float3 x0, float4 w, float h2k,
                                              float nrest)
{
    const float ws = fadd(fadd(w.x, w.y), fadd(w.z, w.w));
    const float3 e = make_float3(ffma(w.y, e1.x, ffma(w.z, e2.x, ffma(w.w, e3.x, fmul(ws, x0.x)))),
                                 ffma(w.y, e1.y, ffma(w.z, e2.y, ffma(w.w, e3.y, fmul(ws, x0.y)))),
                                 ffma(w.y, e1.z, ffma(w.z, e2.z, ffma(w.w, e3.z, fmul(ws, x0.z)))));
    return hinge_q<MODE>(e, h2k, nrest);
}

// The same with a fifth term: the outer corner x of a cell's outer-edge
// hinge, at edge vector ex from x_0 with weight wx.
template <int MODE>
__device__ __forceinline__ float3 hinge_force_x(float3 e1, float3 e2, float3 e3, float3 ex, float3 x0, float4 w,
                                                float wx, float h2k, float nrest)
{
    const float ws = fadd(fadd(fadd(w.x, w.y), fadd(w.z, w.w)), wx);
    const float3 e =
        make_float3(ffma(wx, ex.x, ffma(w.y, e1.x, ffma(w.z, e2.x, ffma(w.w, e3.x, fmul(ws, x0.x))))),
                    ffma(wx, ex.y, ffma(w.y, e1.y, ffma(w.z, e2.y, ffma(w.w, e3.y, fmul(ws, x0.y))))),
                    ffma(wx, ex.z, ffma(w.y, e1.z, ffma(w.z, e2.z, ffma(w.w, e3.z, fmul(ws, x0.z))))));
    return hinge_q<MODE>(e, h2k, nrest);
}

__device__ __forceinline__ float3 edge4(float4 yi, float4 di, float4 yj, float4 dj)
{
    return make_float3(fadd(fsub(yj.x, yi.x), fsub(dj.x, di.x)), fadd(fsub(yj.y, yi.y), fsub(dj.y, di.y)),
                       fadd(fsub(yj.z, yi.z), fsub(dj.z, di.z)));
}

// The six outputs of one cell: o_k for c_k is t0's + t1's contribution, then
// h0's, h1's and h2's (w_k q added by fused multiply-add); o4 / o5 are the
// outer corners' shares of h1 / h2.  Every launch structure calls this, so
// the per-cell sums are bitwise the same everywhere.
template <int MODE>
__device__ __forceinline__ void cell_force(const CellRec& r, const float4* sy, const float4* sd, float3 (&o)[6])
{
    const int i0 = r.c01 & 0xffffu, i1 = r.c01 >> 16, i2 = r.c23 & 0xffffu, i3 = r.c23 >> 16;
    const int j1 = r.x12 & 0xffffu, j2 = r.x12 >> 16;
    const float4 y0 = sy[i0], d0 = sd[i0], y1 = sy[i1], d1 = sd[i1];
    const float4 y2 = sy[i2], d2 = sd[i2], y3 = sy[i3], d3 = sd[i3];
    // an absent outer hinge names c0 as its outer corner: its data are c0's
    // (same values, two fewer shared loads; the packed form below, used by
    // the resident kernel, measured slower with this)
    const float4 yx1 = j1 == i0 ? y0 : sy[j1], dx1 = j1 == i0 ? d0 : sd[j1];
    const float4 yx2 = j2 == i0 ? y0 : sy[j2], dx2 = j2 == i0 ? d0 : sd[j2];
    const float3 e01 = edge4(y0, d0, y1, d1), e02 = edge4(y0, d0, y2, d2), e03 = edge4(y0, d0, y3, d3);
    const float3 e13 = edge4(y1, d1, y3, d3);
    const float3 ex1 = edge4(y0, d0, yx1, dx1), ex2 = edge4(y0, d0, yx2, dx2);
    const float3 x0 = make_float3(fadd(y0.x, d0.x), fadd(y0.y, d0.y), fadd(y0.z, d0.z));
    float3 a0, a1, a2, b0, b1, b3;
    tri_force<MODE>(e01, e02, r.G0, r.h2wA0, a0, a1, a2);
    tri_force<MODE>(make_float3(-e01.x, -e01.y, -e01.z), e13, r.G1, r.h2wA1, b1, b0, b3);
    const float3 q0 = hinge_force<MODE>(e01, e02, e03, x0, r.W0, r.h2k0, r.nrest0);
    const float3 q1 = hinge_force_x<MODE>(e01, e02, e03, ex1, x0, r.W1, r.wx1, r.h2k1, r.nrest1);
    const float3 q2 = hinge_force_x<MODE>(e01, e02, e03, ex2, x0, r.W2, r.wx2, r.h2k2, r.nrest2);
    auto acc = [&](float3 t, float w0, float w1, float w2) {
        return make_float3(ffma(w2, q2.x, ffma(w1, q1.x, ffma(w0, q0.x, t.x))),
                           ffma(w2, q2.y, ffma(w1, q1.y, ffma(w0, q0.y, t.y))),
                           ffma(w2, q2.z, ffma(w1, q1.z, ffma(w0, q0.z, t.z))));
    };
    o[0] = acc(fadd3(a0, b0), r.W0.x, r.W1.x, r.W2.x);
    o[1] = acc(fadd3(a1, b1), r.W0.y, r.W1.y, r.W2.y);
    o[2] = acc(a2, r.W0.z, r.W1.z, r.W2.z);
    o[3] = acc(b3, r.W0.w, r.W1.w, r.W2.w);
    o[4] = scale3(q1, r.wx1);
    o[5] = scale3(q2, r.wx2);
}

// ---------------------------------------------------------------------------
// Packed form of the cell arithmetic: x and y components in one float2 and
// one two-lane instruction (add/mul/fma .f32x2), z alone.  Every lane is
// rounded exactly like the scalar operation it replaces (a - b is formed as
// fma(b, -1, a), which is exact before its single rounding), so the packed
// functions give the bits of the scalar ones above with about a third fewer
// floating-point instructions.
// ---------------------------------------------------------------------------
struct V3 {
    float2 xy;
    float  z;
};
__device__ __forceinline__ float2 bc2(float s) { return make_float2(s, s); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ V3 v3(float4 a) { return V3{make_float2(a.x, a.y), a.z}; }
__device__ __forceinline__ V3 v3(float3 a) { return V3{make_float2(a.x, a.y), a.z}; }
__device__ __forceinline__ float3 f3(V3 a) { return make_float3(a.xy.x, a.xy.y, a.z); }
__device__ __forceinline__ V3 vadd(V3 a, V3 b) { return V3{add2(a.xy, b.xy), fadd(a.z, b.z)}; }
__device__ __forceinline__ V3 vsub(V3 a, V3 b) { return V3{sub2(a.xy, b.xy), fsub(a.z, b.z)}; }
__device__ __forceinline__ V3 vneg(V3 a) { return V3{make_float2(-a.xy.x, -a.xy.y), -a.z}; }
__device__ __forceinline__ V3 vscale(V3 a, float s) { return V3{mul2(a.xy, bc2(s)), fmul(a.z, s)}; }
// a * s + c
__device__ __forceinline__ V3 vfma(V3 a, float s, V3 c) { return V3{fma2(a.xy, bc2(s), c.xy), ffma(a.z, s, c.z)}; }
__device__ __forceinline__ float vdot(V3 a, V3 b) { return ffma(a.xy.x, b.xy.x, ffma(a.xy.y, b.xy.y, fmul(a.z, b.z))); }

// (y_j - y_i) + (d_j - d_i)
__device__ __forceinline__ V3 edge4_p(float4 yi, float4 di, float4 yj, float4 dj)
{
    return vadd(vsub(v3(yj), v3(yi)), vsub(v3(dj), v3(di)));
}

// polar_consistent in packed form
__device__ __forceinline__ void polar_consistent_p(V3 F0, V3 F1, V3& R0, V3& R1)
{
    const float n0sq = vdot(F0, F0);
    const V3 b0 = n0sq > 1e-20f ? vscale(F0, rsqrtf(n0sq)) : V3{make_float2(1.f, 0.f), 0.f};
    const float a01 = vdot(F1, b0);
    const V3 c1 = vfma(b0, -a01, F1);
    const float n1sq = vdot(c1, c1);
    V3 b1;
    if (n1sq > 1e-20f) {
        b1 = vscale(c1, rsqrtf(n1sq));
    } else {   // F1 parallel to F0: any unit vector orthogonal to b0
        float3 q = make_float3(-b0.xy.y, b0.xy.x, 0.f);
        float nq = ffma(q.x, q.x, fmul(q.y, q.y));
        if (nq < 1e-20f) { q = make_float3(0.f, -b0.z, b0.xy.y); nq = ffma(q.y, q.y, fmul(q.z, q.z)); }
        b1 = v3(scale3(q, rsqrtf(nq)));
    }
    const float a00 = vdot(b0, F0), a10 = vdot(b1, F0), a11 = vdot(b1, F1);
    const float s = fadd(a00, a11), t = fsub(a10, a01);
    const float rr = ffma(s, s, fmul(t, t));
    float c = 1.f, sn = 0.f;
    if (rr > 1e-30f) { const float r = rsqrtf(rr); c = fmul(s, r); sn = fmul(t, r); }
    R0 = vfma(b0, c, vscale(b1, sn));
    R1 = vfma(b1, c, vscale(vneg(b0), sn));
}

// tri_force in packed form
template <int MODE>
__device__ __forceinline__ void tri_force_p(V3 d1, V3 d2, float4 G, float h2wA, V3& c0, V3& c1, V3& c2)
{
    const float g00 = G.x, g10 = G.y, g01 = G.z, g11 = G.w;
    const V3 F0 = vfma(d1, g00, vscale(d2, g10));
    const V3 F1 = vfma(d1, g01, vscale(d2, g11));
    V3 q0, q1;
    if (MODE == kModeConsistent) {
        V3 R0, R1;
        polar_consistent_p(F0, F1, R0, R1);
        q0 = vscale(vsub(R0, F0), h2wA);
        q1 = vscale(vsub(R1, F1), h2wA);
    } else {
        float3 R0, R1;
        polar_literal(f3(F0), f3(F1), R0, R1);
        q0 = vscale(v3(R0), h2wA);
        q1 = vscale(v3(R1), h2wA);
    }
    const float s0 = -fadd(g00, g10), s1 = -fadd(g01, g11);
    c0 = vfma(q0, s0, vscale(q1, s1));
    c1 = vfma(q0, g00, vscale(q1, g01));
    c2 = vfma(q0, g10, vscale(q1, g11));
}

// hinge_q in packed form
template <int MODE>
__device__ __forceinline__ V3 hinge_q_p(V3 e, float h2k, float nrest)
{
    if (MODE == kModeConsistent) {
        const float n2 = vdot(e, e);
        V3 p = V3{make_float2(0.f, 0.f), 0.f};
        if (nrest > 1e-10f && n2 > 1e-20f) p = vscale(e, fmul(nrest, rsqrtf(n2)));
        return vscale(vsub(p, e), h2k);
    }
    return v3(hinge_q<MODE>(f3(e), h2k, nrest));
}

// hinge_force / hinge_force_x in packed form (wx = 0 terms absent: x = false)
template <int MODE, bool X>
__device__ __forceinline__ V3 hinge_force_p(V3 e1, V3 e2, V3 e3, V3 ex, V3 x0, float4 w, float wx, float h2k,
                                            float nrest)
{
    float ws = fadd(fadd(w.x, w.y), fadd(w.z, w.w));
    if (X) ws = fadd(ws, wx);
    V3 e = vfma(e1, w.y, vfma(e2, w.z, vfma(e3, w.w, vscale(x0, ws))));
    if (X) e = vfma(ex, wx, e);
    return hinge_q_p<MODE>(e, h2k, nrest);
}

// cell_force in packed form (bitwise the same outputs).  It needs more
// registers at once; the resident kernel, which has them, uses it.
template <int MODE>
__device__ __forceinline__ void cell_force_p(const CellRec& r, const float4* sy, const float4* sd, float3 (&o)[6])
{
    const int i0 = r.c01 & 0xffffu, i1 = r.c01 >> 16, i2 = r.c23 & 0xffffu, i3 = r.c23 >> 16;
    const int j1 = r.x12 & 0xffffu, j2 = r.x12 >> 16;
    const float4 y0 = sy[i0], d0 = sd[i0], y1 = sy[i1], d1 = sd[i1];
    const float4 y2 = sy[i2], d2 = sd[i2], y3 = sy[i3], d3 = sd[i3];
    const float4 yx1 = sy[j1], dx1 = sd[j1], yx2 = sy[j2], dx2 = sd[j2];
    const V3 e01 = edge4_p(y0, d0, y1, d1), e02 = edge4_p(y0, d0, y2, d2), e03 = edge4_p(y0, d0, y3, d3);
    const V3 e13 = edge4_p(y1, d1, y3, d3);
    const V3 ex1 = edge4_p(y0, d0, yx1, dx1), ex2 = edge4_p(y0, d0, yx2, dx2);
    const V3 x0 = vadd(v3(y0), v3(d0));
    V3 a0, a1, a2, b0, b1, b3;
    tri_force_p<MODE>(e01, e02, r.G0, r.h2wA0, a0, a1, a2);
    tri_force_p<MODE>(vneg(e01), e13, r.G1, r.h2wA1, b1, b0, b3);
    const V3 q0 = hinge_force_p<MODE, false>(e01, e02, e03, e03, x0, r.W0, 0.f, r.h2k0, r.nrest0);
    const V3 q1 = hinge_force_p<MODE, true>(e01, e02, e03, ex1, x0, r.W1, r.wx1, r.h2k1, r.nrest1);
    const V3 q2 = hinge_force_p<MODE, true>(e01, e02, e03, ex2, x0, r.W2, r.wx2, r.h2k2, r.nrest2);
    // t + w0 q0 + w1 q1 + w2 q2, in that order
    auto acc = [&](V3 t, float w0, float w1, float w2) { return vfma(q2, w2, vfma(q1, w1, vfma(q0, w0, t))); };
    o[0] = f3(acc(vadd(a0, b0), r.W0.x, r.W1.x, r.W2.x));
    o[1] = f3(acc(vadd(a1, b1), r.W0.y, r.W1.y, r.W2.y));
    o[2] = f3(acc(a2, r.W0.z, r.W1.z, r.W2.z));
    o[3] = f3(acc(b3, r.W0.w, r.W1.w, r.W2.w));
    o[4] = f3(vscale(q1, r.wx1));
    o[5] = f3(vscale(q2, r.wx2));
}

// Record c of the patch whose records start at `base`, in the device format
// (pdg_layout.h): its nine 16-byte pieces lie kCellGroup pieces apart, so
// the lanes of a warp that load consecutive records read whole lines.  Each
// line is used by one load, so the loads do not allocate in L1 (batch sweep
// 176.3 -> 174.3 us; evict_first: 175.2 us).
__device__ __forceinline__ uint4 ld_nc_na(const uint4* a)
{
    uint4 v;
    asm("ld.global.nc.L1::no_allocate.v4.u32 {%0, %1, %2, %3}, [%4];"
        : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
        : "l"(a));
    return v;
}

__device__ __forceinline__ CellRec load_cell(const CellRec* __restrict__ base, int c)
{
    static_assert(sizeof(CellRec) == 9 * 16, "CellRec is nine 16-byte pieces");
    const uint4* p = reinterpret_cast<const uint4*>(base) + (c / kCellGroup) * (9 * kCellGroup) + (c % kCellGroup);
    const uint4 q0 = ld_nc_na(p), q1 = ld_nc_na(p + kCellGroup), q2 = ld_nc_na(p + 2 * kCellGroup);
    const uint4 q3 = ld_nc_na(p + 3 * kCellGroup), q4 = ld_nc_na(p + 4 * kCellGroup);
    const uint4 q5 = ld_nc_na(p + 5 * kCellGroup), q6 = ld_nc_na(p + 6 * kCellGroup);
    const uint4 q7 = ld_nc_na(p + 7 * kCellGroup), q8 = ld_nc_na(p + 8 * kCellGroup);
    auto f4 = [](uint4 q) {
        return make_float4(__uint_as_float(q.x), __uint_as_float(q.y), __uint_as_float(q.z), __uint_as_float(q.w));
    };
    CellRec r;
    r.G0 = f4(q0); r.G1 = f4(q1); r.W0 = f4(q2); r.W1 = f4(q3); r.W2 = f4(q4);
    r.h2wA0 = __uint_as_float(q5.x); r.h2wA1 = __uint_as_float(q5.y);
    r.h2k0 = __uint_as_float(q5.z); r.nrest0 = __uint_as_float(q5.w);
    r.h2k1 = __uint_as_float(q6.x); r.nrest1 = __uint_as_float(q6.y);
    r.wx1 = __uint_as_float(q6.z); r.h2k2 = __uint_as_float(q6.w);
    r.nrest2 = __uint_as_float(q7.x); r.wx2 = __uint_as_float(q7.y);
    r.c01 = q7.z; r.c23 = q7.w;
    r.x12 = q8.x; r.vm01 = q8.y; r.vm23 = q8.z; r.vm45 = q8.w;
    return r;
}

// Vertex-major slots (every sweep kernel): the record carries each
// output's slot address (0xffff for a halo corner or an absent output).  A
// slot holds its contribution as an (x, y) pair in cxy and z in cz: two
// shared-memory accesses per slot.
template <int MODE>
__device__ __forceinline__ void cell_contrib_vm(const CellRec& r, const float4* sy, const float4* sd, float2* cxy,
                                                float* cz)
{
    float3 o[6];
    cell_force<MODE>(r, sy, sd, o);
    const uint32_t vm[6] = {r.vm01 & 0xffffu, r.vm01 >> 16, r.vm23 & 0xffffu, r.vm23 >> 16,
                            r.vm45 & 0xffffu, r.vm45 >> 16};
    #pragma unroll
    for (int k = 0; k < 6; ++k)
        if (vm[k] != 0xffffu) { cxy[vm[k]] = make_float2(o[k].x, o[k].y); cz[vm[k]] = o[k].z; }
}

// Vertex-major slots with the packed cell arithmetic (same bits).
template <int MODE>
__device__ __forceinline__ void cell_contrib_vm_p(const CellRec& r, const float4* sy, const float4* sd, float2* cxy,
                                                  float* cz)
{
    float3 o[6];
    cell_force_p<MODE>(r, sy, sd, o);
    const uint32_t vm[6] = {r.vm01 & 0xffffu, r.vm01 >> 16, r.vm23 & 0xffffu, r.vm23 >> 16,
                            r.vm45 & 0xffffu, r.vm45 >> 16};
    #pragma unroll
    for (int k = 0; k < 6; ++k)
        if (vm[k] != 0xffffu) { cxy[vm[k]] = make_float2(o[k].x, o[k].y); cz[vm[k]] = o[k].z; }
}

template <int MODE>
__device__ __forceinline__ void hinge_contrib_vm(const HingeRec& r, uint2 hs, const float4* sy, const float4* sd,
                                                 float2* cxy, float* cz)
{
    const int i0 = r.l01 & 0xffffu, i1 = r.l01 >> 16, i2 = r.l23 & 0xffffu, i3 = r.l23 >> 16;
    const float4 y0 = sy[i0], d0 = sd[i0];
    const float3 x0 = make_float3(fadd(y0.x, d0.x), fadd(y0.y, d0.y), fadd(y0.z, d0.z));
    const float4 w = r.w;
    const float3 q = hinge_force<MODE>(edge(sy, sd, i0, i1), edge(sy, sd, i0, i2), edge(sy, sd, i0, i3), x0, w,
                                       r.h2k, r.nrest);
    const uint32_t s0 = hs.x & 0xffffu, s1 = hs.x >> 16, s2 = hs.y & 0xffffu, s3 = hs.y >> 16;
    if (s0 != 0xffffu) { cxy[s0] = make_float2(fmul(w.x, q.x), fmul(w.x, q.y)); cz[s0] = fmul(w.x, q.z); }
    if (s1 != 0xffffu) { cxy[s1] = make_float2(fmul(w.y, q.x), fmul(w.y, q.y)); cz[s1] = fmul(w.y, q.z); }
    if (s2 != 0xffffu) { cxy[s2] = make_float2(fmul(w.z, q.x), fmul(w.z, q.y)); cz[s2] = fmul(w.z, q.z); }
    if (s3 != 0xffffu) { cxy[s3] = make_float2(fmul(w.w, q.x), fmul(w.w, q.y)); cz[s3] = fmul(w.w, q.z); }
}

// The force on an owned vertex is defined as (sum of the first half of its
// contributions) + (sum of the second half), the first half holding
// ceil(deg/2) of them, each half in the canonical order (the cloth's cells,
// then its lone hinges).  Every kernel forms exactly this, so
// one that gives the two halves to two threads produces the same bits.
__device__ __forceinline__ int gather_half(int deg) { return (deg + 1) >> 1; }
// vertex-major slots: contribution j of vertex l at j*npad + l
__device__ __forceinline__ float3 gather_vm(int l, int j0, int j1, int npad, const float2* cxy, const float* cz)
{
    float fx = 0.f, fy = 0.f, fz = 0.f;
    for (int j = j0, s = j0 * npad + l; j < j1; ++j, s += npad) {
        const float2 v = cxy[s];
        fx = fadd(fx, v.x); fy = fadd(fy, v.y); fz = fadd(fz, cz[s]);
    }
    return make_float3(fx, fy, fz);
}

// gather_vm for at most M contributions: every slot load is issued before
// the additions, which run in the same order (same bits).
template <int M>
__device__ __forceinline__ float3 gather_vm_u(int l, int j0, int j1, int npad, const float2* cxy, const float* cz)
{
    float2 vxy[M];
    float vz[M];
    #pragma unroll
    for (int i = 0; i < M; ++i) {
        const bool ok = j0 + i < j1;
        const int s = ok ? (j0 + i) * npad + l : l;   // always inside the slot arrays
        vxy[i] = cxy[s]; vz[i] = cz[s];
    }
    float fx = 0.f, fy = 0.f, fz = 0.f;
    #pragma unroll
    for (int i = 0; i < M; ++i)
        if (j0 + i < j1) { fx = fadd(fx, vxy[i].x); fy = fadd(fy, vxy[i].y); fz = fadd(fz, vz[i]); }
    return make_float3(fx, fy, fz);
}

// gather_vm_u with the loads past the vertex's contributions predicated off
// instead of re-reading an in-range slot: fewer shared-memory wavefronts,
// same sums.  The streaming sweep uses it (batch sweep 199.5 -> 196.8 us);
// in the resident kernel it measured 0.7 % slower, so that keeps gather_vm_u.
template <int M>
__device__ __forceinline__ float3 gather_vm_p(int l, int j0, int j1, int npad, const float2* cxy, const float* cz)
{
    float2 vxy[M];
    float vz[M];
    #pragma unroll
    for (int i = 0; i < M; ++i) {
        vxy[i] = make_float2(0.f, 0.f);
        vz[i] = 0.f;
        if (j0 + i < j1) { const int s = (j0 + i) * npad + l; vxy[i] = cxy[s]; vz[i] = cz[s]; }
    }
    float fx = 0.f, fy = 0.f, fz = 0.f;
    #pragma unroll
    for (int i = 0; i < M; ++i)
        if (j0 + i < j1) { fx = fadd(fx, vxy[i].x); fy = fadd(fy, vxy[i].y); fz = fadd(fz, vz[i]); }
    return make_float3(fx, fy, fz);
}

// Jacobi update of one owned vertex in the consistent form:
// -r = f - m d;  d_hat = d + gamma D^-1 (-r);  d' = omega (d_hat - d_prev) + d_prev.
__device__ __forceinline__ float4 update_consistent(float4 d, float4 y, float3 f, float4 dp, float gamma,
                                                   float omega, float& r2)
{
    const float rx = fsub(f.x, fmul(y.w, d.x));
    const float ry = fsub(f.y, fmul(y.w, d.y));
    const float rz = fsub(f.z, fmul(y.w, d.z));
    float4 o = d;
    r2 = 0.f;
    if (d.w >= 0.f) {   // free vertex (pinned ones carry -1)
        r2 = ffma(rx, rx, ffma(ry, ry, fmul(rz, rz)));
        const float gi = fmul(gamma, d.w);
        o.x = ffma(omega, fsub(ffma(gi, rx, d.x), dp.x), dp.x);
        o.y = ffma(omega, fsub(ffma(gi, ry, d.y), dp.y), dp.y);
        o.z = ffma(omega, fsub(ffma(gi, rz, d.z), dp.z), dp.z);
    }
    return o;
}

// x = rhs / diag with rhs = m y + f (src/pd_solver.cu:371-398), stored as x - y.
__device__ __forceinline__ float4 update_literal(float4 d, float4 y, float3 f)
{
    float4 o = d;
    if (d.w >= 0.f) {
        o.x = fsub(fmul(fadd(f.x, fmul(y.w, y.x)), d.w), y.x);
        o.y = fsub(fmul(fadd(f.y, fmul(y.w, y.y)), d.w), y.y);
        o.z = fsub(fmul(fadd(f.z, fmul(y.w, y.z)), d.w), y.z);
    }
    return o;
}

__device__ __forceinline__ float warp_sum(float v)
{
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum of r2 added to the per-sweep accumulator (one double atomic
// per block).  Contains a __syncthreads.
template <int NT>
__device__ __forceinline__ void block_residual(float r2, float* red, double* acc)
{
    const int tid = threadIdx.x;
    r2 = warp_sum(r2);
    if ((tid & 31) == 0) red[tid >> 5] = r2;
    __syncthreads();
    if (tid < 32) {
        float v = tid < NT / 32 ? red[tid] : 0.f;
        v = warp_sum(v);
        if (tid == 0) atomicAdd(acc, (double)v);
    }
}

// ---------------------------------------------------------------------------
// Fused sweep over one patch.  `k` is the sweep index: the block reads the
// offsets d^k = x^k - y from buf[k & 1], reads d^(k-1) and writes d^(k+1) in
// buf[(k+1) & 1] (the same slot, owned by this thread), and adds
// ||r(x^k)||^2 to acc[cloth][k].  With res_only it only evaluates the
// residual.  Data produced by other blocks is loaded with __ldcg (L2, not L1),
// so the same code is correct inside the persistent kernel between grid
// barriers.  Shared memory: sy, sd (float4 per local vertex), then the three
// slot arrays in vertex-major order (ph.vm_nslot each).
// ---------------------------------------------------------------------------
template <int MODE, int NT>
__device__ __forceinline__ void process_patch(const IterArgs& a, const PatchHdr& ph, int k, bool res_only,
                                              float omega, float4* sy, float2* cxy, float* cz,
                                              float* red, const int* skip_s = nullptr,
                                              const float* omega_s = nullptr)
{
    // select, not index: a dynamic index into the parameter struct would
    // copy it to local memory
    const float4* __restrict__ Dk = (k & 1) ? a.buf[1] : a.buf[0];
    float4* __restrict__ Dn = (k & 1) ? a.buf[0] : a.buf[1];
    float4* sd = sy + ph.nlocal;
    const int tid = threadIdx.x;

    const int nlocal = ph.nlocal, nown = ph.nown, vbegin = ph.vbegin;
    const int* __restrict__ halo = a.halo + ph.halo_off - nown;   // halo list, indexed by local vertex
    const int* __restrict__ cp = a.csr_ptr + ph.csr_off;
    const CellRec* __restrict__ cr = a.cells + ph.cell_off;
    const int ncell = ph.ncell, nhin = ph.nhinge;

    // 0. loads issued before the staging barrier, so that their memory round
    // trips overlap the staging: the gather pointers and d^(k-1) of this
    // thread's first owned vertex.  (Loading its first cell record here too
    // costs more in register spills than it saves.)
    int cp0 = 0, cp1 = 0;
    float4 dp0 = make_float4(0.f, 0.f, 0.f, 0.f);
    if (tid < nown) {
        cp0 = __ldg(&cp[tid]);
        cp1 = __ldg(&cp[tid + 1]);
        if (MODE == kModeConsistent && !res_only) dp0 = __ldcg(&Dn[vbegin + tid]);
    }

    // 1. stage y and d^k of owned + halo vertices, two per thread and pass
    // with both index loads issued before the position loads
    for (int l0 = tid; l0 < nlocal; l0 += 2 * NT) {
        const int l1 = l0 + NT;
        const bool has1 = l1 < nlocal;
        const int l1c = has1 ? l1 : l0;
        const int g0 = l0 < nown ? vbegin + l0 : __ldg(&halo[l0]);
        const int g1 = l1c < nown ? vbegin + l1c : __ldg(&halo[l1c]);
        const float4 y0 = __ldcg(&a.Y[g0]), d0 = __ldcg(&Dk[g0]);
        const float4 y1 = __ldcg(&a.Y[g1]), d1 = __ldcg(&Dk[g1]);
        sy[l0] = y0;
        sd[l0] = d0;
        if (has1) { sy[l1] = y1; sd[l1] = d1; }
    }
    __syncthreads();
    // a skip decision and weight taken by thread 0 while the block staged
    if (skip_s && *(const volatile int*)skip_s) return;
    if (omega_s) omega = *(const volatile float*)omega_s;

    // 2. local step: cells then lone hinges, contributions to shared slots
    for (int c = tid; c < ncell; c += NT) {
        const CellRec r = load_cell(cr, c);
        cell_contrib_vm<MODE>(r, sy, sd, cxy, cz);
    }
    const HingeRec* __restrict__ hr = a.hinges + ph.hinge_off;
    const uint2* __restrict__ hv = a.hvm + ph.hinge_off;
    for (int e = tid; e < nhin; e += NT) {
        const HingeRec r = hr[e];
        hinge_contrib_vm<MODE>(r, __ldg(&hv[e]), sy, sd, cxy, cz);
    }
    __syncthreads();

    // 3. global step per owned vertex
    const float gamma = a.cinfo[ph.cloth].gamma;
    const int npad = ph.vm_npad;
    float r2 = 0.f;
    for (int l = tid; l < nown; l += NT) {
        // contributions j = 0..deg-1 of vertex l: first half + second half
        const bool first = l == tid;
        const int deg = first ? cp1 - cp0 : __ldg(&cp[l + 1]) - __ldg(&cp[l]);
        const int h = gather_half(deg);
        const float3 f = fadd3(gather_vm(l, 0, h, npad, cxy, cz), gather_vm(l, h, deg, npad, cxy, cz));
        const int g = vbegin + l;
        const float4 d = sd[l];
        const float4 y = sy[l];
        if (MODE == kModeConsistent) {
            float rv;
            const float4 dp = res_only ? d : (first ? dp0 : __ldcg(&Dn[g]));
            const float4 o = update_consistent(d, y, f, dp, gamma, omega, rv);
            r2 += rv;
            if (!res_only) Dn[g] = o;
        } else if (!res_only) {
            Dn[g] = update_literal(d, y, f);
        }
    }
    if (MODE == kModeConsistent) block_residual<NT>(r2, red, a.acc + (size_t)ph.cloth * a.acc_stride + k);
}

// Loads that are issued in program order and not moved past later branches
// (asm volatile): a chain of dependent decisions then waits for one memory
// round trip instead of one per condition.
__device__ __forceinline__ int ld_cg_s32(const int* p)
{
    int v;
    asm volatile("ld.global.cg.s32 %0, [%1];" : "=r"(v) : "l"(__cvta_generic_to_global(p)));
    return v;
}
__device__ __forceinline__ double ld_cg_f64(const double* p)
{
    double v;
    asm volatile("ld.global.cg.f64 %0, [%1];" : "=d"(v) : "l"(__cvta_generic_to_global(p)));
    return v;
}

// Per-cloth decision at the start of sweep k, taken by one thread per block;
// every block of a cloth reaches the same answer from the same data.
// Returns true if the cloth is done.  The cloth's first patch records it.
// With check == false only the static cap is applied (the per-sweep sums may
// still be incomplete: sweeps synchronised with neighbours only).  Every
// value it may need is loaded up front.
__device__ __forceinline__ bool cloth_done(const IterArgs& a, int c, int k, bool designated, bool check = true)
{
    ClothRT* rt = a.crt + c;
    const ClothInfo& ci = a.cinfo[c];
    const double* acc = a.acc + (size_t)c * a.acc_stride;
    const int active = ld_cg_s32(&rt->active);
    const double acc0 = ld_cg_f64(&acc[0]);
    const double rk2 = ld_cg_f64(&acc[k >= 1 ? k - 1 : 0]);      // ||r(x^(k-1))||^2
    const double ry2_rt = ld_cg_f64(&rt->res_y2);
    const int mode = ci.mode, init = ci.init, max_iter = ci.max_iter;
    const float tol = ci.tol;
    if (!active) return true;
    if (check && k >= 1 && mode == kModeConsistent) {
        // normaliser: the residual of the inertial start, measured by the
        // warm-start selection when a learned start was evaluated, else the
        // residual of the start iterate itself
        const bool own_start = !(init >= 2 && a.warm_active);
        const double ry2 = (k == 1 && own_start) ? acc0 : ry2_rt;
        if (k == 1 && designated) {
            rt->res0_2 = acc0;
            if (own_start) rt->res_y2 = acc0;
        }
        if (!isfinite(rk2)) {
            if (designated) { rt->status = -6; rt->used = k - 1; rt->resf_2 = rk2; rt->active = 0; }
            return true;
        }
        if (tol > 0.f && rk2 <= (double)tol * (double)tol * ry2) {
            if (designated) { rt->used = k - 1; rt->resf_2 = rk2; rt->active = 0; }
            return true;
        }
        if (k > max_iter) {   // this cloth's cap: x^max_iter and its residual are final
            if (designated) { rt->used = max_iter; rt->resf_2 = rk2; rt->active = 0; }
            return true;
        }
    }
    if (k >= max_iter && (k > max_iter || !a.have_final)) {
        if (designated && (check || mode != kModeConsistent)) {
            rt->used = max_iter; rt->resf_2 = -1.0; rt->active = 0;
        }
        return true;
    }
    return false;
}

// Start of a frame: the cloth's record and per-sweep sums are cleared.
__device__ __forceinline__ void reset_rt(ClothRT* crt, double* acc, int acc_stride, int c, int t0, int nt)
{
    if (t0 == 0) {
        ClothRT r;
        r.active = 1; r.used = 0; r.status = 0; r.warm = 0;
        r.res_y2 = 0.0; r.res0_2 = 0.0; r.resf_2 = -1.0;
        crt[c] = r;
    }
    for (int k = t0; k < acc_stride; k += nt) acc[(size_t)c * acc_stride + k] = 0.0;
}

// y = x + h v + h^2 a (w = mass); start offset d^0 = x^0 - y into both
// buffers (w = inverse diagonal, -1 for pinned vertices).
__device__ __forceinline__ void predict_vertex_xv(int i, float4 x, float4 v, const float4* aux, const float* mass,
                                                  const int* vcloth, const ClothInfo* cinfo, const float4* warm,
                                                  float4* Y, float4* A, float4* B)
{
    const ClothInfo& ci = cinfo[vcloth[i]];
    const float h = ci.h, h2 = fmul(h, h);
    const float4 au = __ldcg(&aux[i]);
    float4 y;
    y.x = ffma(h2, ci.ext[0], ffma(h, v.x, x.x));
    y.y = ffma(h2, ci.ext[1], ffma(h, v.y, x.y));
    y.z = ffma(h2, ci.ext[2], ffma(h, v.z, x.z));
    y.w = mass[i];
    Y[i] = y;
    float4 s;
    if (au.w < 0.f)                    s = make_float4(fsub(au.x, y.x), fsub(au.y, y.y), fsub(au.z, y.z), au.w);
    else if (ci.init == 1)             s = make_float4(fsub(x.x, y.x), fsub(x.y, y.y), fsub(x.z, y.z), au.w);
    else if (ci.init >= 2 && warm) {   const float4 w = __ldcg(&warm[i]); s = make_float4(w.x, w.y, w.z, au.w); }
    else                               s = make_float4(0.f, 0.f, 0.f, au.w);
    A[i] = s;
    B[i] = s;
}

__device__ __forceinline__ void predict_vertex(int i, const float4* X, const float4* V, const float4* aux,
                                               const float* mass, const int* vcloth, const ClothInfo* cinfo,
                                               const float4* warm, float4* Y, float4* A, float4* B)
{
    predict_vertex_xv(i, __ldcg(&X[i]), __ldcg(&V[i]), aux, mass, vcloth, cinfo, warm, Y, A, B);
}

// Cloths still active after the last sweep keep x^max_iter.  A non-finite
// per-sweep sum marks the cloth as failed (sweeps that ran with neighbour
// synchronisation skip the per-sweep check).
__device__ __forceinline__ void frame_stats_cloth(const IterArgs& a, int c)
{
    ClothRT* rt = a.crt + c;
    const ClothInfo& ci = a.cinfo[c];
    const double* acc = a.acc + (size_t)c * a.acc_stride;
    if (ci.mode == kModeConsistent) {
        rt->res0_2 = __ldcg(&acc[0]);
        if (!(ci.init >= 2 && a.warm_active)) rt->res_y2 = rt->res0_2;
    }
    if (__ldcg(&rt->active)) {
        rt->used = ci.max_iter;
        if (ci.mode == kModeConsistent) {
            bool finite = true;
            for (int k = 0; k <= ci.max_iter && k < a.acc_stride; ++k) finite = finite && isfinite(__ldcg(&acc[k]));
            const double rf = __ldcg(&acc[ci.max_iter]);
            rt->resf_2 = a.have_final ? rf : -1.0;
            if (!finite) rt->status = -6;
        } else {
            rt->resf_2 = -1.0;
        }
        rt->active = 0;
    }
}

// x = y + d^used; v = (x - x_n)(1 - damping)/h, formed without cancellation
// as (1 - damping)(v_n + h a + d/h) since x - x_n = h v_n + h^2 a + d.
// Pins go to their target with v = 0.  A cloth whose solve produced
// NaN/Inf keeps x_n and gets v = 0.
__device__ __forceinline__ void finalize_vertex(int i, float4* X, float4* V, const float4* Y, const float4* A,
                                                const float4* B, const float4* aux, const int* vcloth,
                                                const ClothInfo* cinfo, const ClothRT* crt)
{
    const int c = vcloth[i];
    const ClothInfo& ci = cinfo[c];
    const int status = __ldcg(&crt[c].status);
    const int used = __ldcg(&crt[c].used);
    const float4 au = __ldcg(&aux[i]);
    if (au.w < 0.f) {
        X[i] = make_float4(au.x, au.y, au.z, 0.f);
        V[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    if (status != 0) {
        V[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const float4 d = (used & 1) ? __ldcg(&B[i]) : __ldcg(&A[i]);
    const float4 y = __ldcg(&Y[i]);
    const float4 v = __ldcg(&V[i]);
    const float h = ci.h, sc = 1.f - ci.damping, ih = fdiv(1.f, h);
    V[i] = make_float4(fmul(sc, ffma(d.x, ih, ffma(h, ci.ext[0], v.x))), fmul(sc, ffma(d.y, ih, ffma(h, ci.ext[1], v.y))),
                       fmul(sc, ffma(d.z, ih, ffma(h, ci.ext[2], v.z))), 0.f);
    X[i] = make_float4(fadd(y.x, d.x), fadd(y.y, d.y), fadd(y.z, d.z), 0.f);
}

}  // namespace pdg
