// Device-side pieces of the PD solve shared by the per-iteration kernel and
// the persistent kernel.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "pdg_layout.h"

namespace pdg {

enum { kModeConsistent = 0, kModeLiteral = 1 };

// ---------------------------------------------------------------------------
// Stretch projection, consistent form: Gram-Schmidt basis (b0, b1) of F's
// columns, F2d = [b0 b1]^T F, closest rotation in SO(2) in closed form
// R2d = rot(atan2(F2d10 - F2d01, F2d00 + F2d11)), R = [b0 b1] R2d.  This is
// the projection of src/stretch_reference.cpp:38-68 (JacobiSVD U V^T with the
// determinant fix) without the SVD.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void polar_consistent(float3 F0, float3 F1, float3& R0, float3& R1)
{
    const float n0sq = F0.x * F0.x + F0.y * F0.y + F0.z * F0.z;
    float3 b0;
    if (n0sq > 1e-20f) {
        const float r = rsqrtf(n0sq);
        b0 = make_float3(F0.x * r, F0.y * r, F0.z * r);
    } else {
        b0 = make_float3(1.f, 0.f, 0.f);
    }
    const float a01 = F1.x * b0.x + F1.y * b0.y + F1.z * b0.z;
    const float3 c1 = make_float3(F1.x - a01 * b0.x, F1.y - a01 * b0.y, F1.z - a01 * b0.z);
    const float n1sq = c1.x * c1.x + c1.y * c1.y + c1.z * c1.z;
    float3 b1;
    if (n1sq > 1e-20f) {
        const float r = rsqrtf(n1sq);
        b1 = make_float3(c1.x * r, c1.y * r, c1.z * r);
    } else {
        float3 q = make_float3(-b0.y, b0.x, 0.f);
        float nq = q.x * q.x + q.y * q.y;
        if (nq < 1e-20f) { q = make_float3(0.f, -b0.z, b0.y); nq = q.y * q.y + q.z * q.z; }
        const float r = rsqrtf(nq);
        b1 = make_float3(q.x * r, q.y * r, q.z * r);
    }
    const float a00 = b0.x * F0.x + b0.y * F0.y + b0.z * F0.z;
    const float a10 = b1.x * F0.x + b1.y * F0.y + b1.z * F0.z;
    const float a11 = b1.x * F1.x + b1.y * F1.y + b1.z * F1.z;
    const float s = a00 + a11, t = a10 - a01;
    const float rr = s * s + t * t;
    float c = 1.f, sn = 0.f;
    if (rr > 1e-30f) { const float r = rsqrtf(rr); c = s * r; sn = t * r; }
    R0 = make_float3(b0.x * c + b1.x * sn, b0.y * c + b1.y * sn, b0.z * c + b1.z * sn);
    R1 = make_float3(b1.x * c - b0.x * sn, b1.y * c - b0.y * sn, b1.z * c - b0.z * sn);
}

// ---------------------------------------------------------------------------
// Stretch projection with the semantics of the reference kernel
// tri_stretch_project_kernel (src/pd_solver.cu:48-208): eigenvectors V of
// F2d^T F2d, W = F2d V / sigma, R2d = V W^T (the transpose of the polar
// rotation), R = U R2d.  Used only by the reference-literal mode.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void polar_literal(float3 F0, float3 F1, float3& R0, float3& R1)
{
    const float lf0 = sqrtf(F0.x * F0.x + F0.y * F0.y + F0.z * F0.z);
    float3 u1 = lf0 > 1e-10f ? make_float3(F0.x / lf0, F0.y / lf0, F0.z / lf0) : make_float3(1.f, 0.f, 0.f);
    const float f1u1 = F1.x * u1.x + F1.y * u1.y + F1.z * u1.z;
    const float3 up = make_float3(F1.x - f1u1 * u1.x, F1.y - f1u1 * u1.y, F1.z - f1u1 * u1.z);
    const float lup = sqrtf(up.x * up.x + up.y * up.y + up.z * up.z);
    float3 u2;
    if (lup > 1e-10f) {
        u2 = make_float3(up.x / lup, up.y / lup, up.z / lup);
    } else {
        u2 = fabsf(u1.x) > 0.9f ? make_float3(-u1.y, u1.x, 0.f) : make_float3(0.f, -u1.z, u1.y);
        const float l = sqrtf(u2.x * u2.x + u2.y * u2.y + u2.z * u2.z);
        u2 = make_float3(u2.x / l, u2.y / l, u2.z / l);
    }
    const float F00 = u1.x * F0.x + u1.y * F0.y + u1.z * F0.z;
    const float F01 = u1.x * F1.x + u1.y * F1.y + u1.z * F1.z;
    const float F10 = u2.x * F0.x + u2.y * F0.y + u2.z * F0.z;
    const float F11 = u2.x * F1.x + u2.y * F1.y + u2.z * F1.z;
    const float A00 = F00 * F00 + F10 * F10, A01 = F00 * F01 + F10 * F11, A11 = F01 * F01 + F11 * F11;
    const float tr = (A00 + A11) * 0.5f;
    const float disc = sqrtf(fmaxf(0.f, (A00 - A11) * (A00 - A11) * 0.25f + A01 * A01));
    const float l1 = tr + disc, l2 = tr - disc;
    float v1x = 1.f, v1y = 0.f, v2x = 0.f, v2y = 1.f;
    if (!(disc < 1e-10f || fabsf(A01) < 1e-10f)) {
        const float tmp = l1 - A00;
        const float l = sqrtf(A01 * A01 + tmp * tmp);
        if (l > 1e-10f) { v1x = A01 / l; v1y = tmp / l; }
        v2x = -v1y; v2y = v1x;
    }
    const float s1 = sqrtf(fmaxf(0.f, l1)), s2 = sqrtf(fmaxf(0.f, l2));
    float w1x = 1.f, w1y = 0.f, w2x, w2y;
    if (s1 > 1e-10f) { w1x = (F00 * v1x + F01 * v1y) / s1; w1y = (F10 * v1x + F11 * v1y) / s1; }
    if (s2 > 1e-10f) {
        w2x = (F00 * v2x + F01 * v2y) / s2; w2y = (F10 * v2x + F11 * v2y) / s2;
    } else {
        const float fx = F00 * v2x + F01 * v2y, fy = F10 * v2x + F11 * v2y;
        const float d = w1x * fx + w1y * fy;
        const float wx = fx - d * w1x, wy = fy - d * w1y;
        const float l = sqrtf(wx * wx + wy * wy);
        if (l > 1e-10f) { w2x = wx / l; w2y = wy / l; } else { w2x = -w1y; w2y = w1x; }
    }
    const float r00 = v1x * w1x + v2x * w2x, r01 = v1x * w1y + v2x * w2y;
    const float r10 = v1y * w1x + v2y * w2x, r11 = v1y * w1y + v2y * w2y;
    R0 = make_float3(u1.x * r00 + u2.x * r10, u1.y * r00 + u2.y * r10, u1.z * r00 + u2.z * r10);
    R1 = make_float3(u1.x * r01 + u2.x * r11, u1.y * r01 + u2.y * r11, u1.z * r01 + u2.z * r11);
}

__device__ __forceinline__ float3 f3(float4 a) { return make_float3(a.x, a.y, a.z); }

// Positions are carried as x = y + d: y the inertial prediction, d the
// offset the solve iterates on.  Edge vectors are formed as
// (y_j - y_i) + (d_j - d_i), so their rounding error is that of the small
// offsets, not of coordinates of size ~1 m.
__device__ __forceinline__ float3 edge(const float4* sy, const float4* sd, int i, int j)
{
    const float4 yi = sy[i], yj = sy[j], di = sd[i], dj = sd[j];
    return make_float3((yj.x - yi.x) + (dj.x - di.x), (yj.y - yi.y) + (dj.y - di.y), (yj.z - yi.z) + (dj.z - di.z));
}

// Triangle phase for one local triangle: writes the contributions of its
// three corners to the slots 3*lt + corner.
// Slots are corner-major (corner c of local triangle lt at c*ntri + lt), so
// a warp's stores are unit-stride and free of bank conflicts.
template <int MODE>
__device__ __forceinline__ void triangle_contrib(const TriRec& r, const float4* sy, const float4* sd, int lt,
                                                 int ntri, float* cx, float* cy, float* cz)
{
    const int i0 = r.l01 & 0xffffu, i1 = r.l01 >> 16, i2 = r.l2;
    const float g00 = r.G.x, g10 = r.G.y, g01 = r.G.z, g11 = r.G.w;
    const float3 d1 = edge(sy, sd, i0, i1);
    const float3 d2 = edge(sy, sd, i0, i2);
    const float3 F0 = make_float3(d1.x * g00 + d2.x * g10, d1.y * g00 + d2.y * g10, d1.z * g00 + d2.z * g10);
    const float3 F1 = make_float3(d1.x * g01 + d2.x * g11, d1.y * g01 + d2.y * g11, d1.z * g01 + d2.z * g11);
    float3 R0, R1, q0, q1;
    if (MODE == kModeConsistent) {
        polar_consistent(F0, F1, R0, R1);
        q0 = make_float3(r.h2wA * (R0.x - F0.x), r.h2wA * (R0.y - F0.y), r.h2wA * (R0.z - F0.z));
        q1 = make_float3(r.h2wA * (R1.x - F1.x), r.h2wA * (R1.y - F1.y), r.h2wA * (R1.z - F1.z));
    } else {
        polar_literal(F0, F1, R0, R1);
        q0 = make_float3(r.h2wA * R0.x, r.h2wA * R0.y, r.h2wA * R0.z);
        q1 = make_float3(r.h2wA * R1.x, r.h2wA * R1.y, r.h2wA * R1.z);
    }
    const float s0 = -(g00 + g10), s1 = -(g01 + g11);
    const int b1 = ntri + lt, b2 = 2 * ntri + lt;
    cx[lt] = s0 * q0.x + s1 * q1.x;   cy[lt] = s0 * q0.y + s1 * q1.y;   cz[lt] = s0 * q0.z + s1 * q1.z;
    cx[b1] = g00 * q0.x + g01 * q1.x; cy[b1] = g00 * q0.y + g01 * q1.y; cz[b1] = g00 * q0.z + g01 * q1.z;
    cx[b2] = g10 * q0.x + g11 * q1.x; cy[b2] = g10 * q0.y + g11 * q1.y; cz[b2] = g10 * q0.z + g11 * q1.z;
}

// Hinge phase: e = sum w_i x_i, target p = e * n_rest / |e| (0 if |e| or
// n_rest <= 1e-10, src/pd_solver.cu:304-335); slot s gets h^2 k w_s (p - e)
// (consistent) or h^2 k w_s p (literal).
// Slot s of local hinge e sits at hbase + s*nhin + e.
template <int MODE>
__device__ __forceinline__ void hinge_contrib(const HingeRec& r, const float4* sy, const float4* sd, int e_,
                                              int hbase, int nhin, float* cx, float* cy, float* cz)
{
    // e = sum w_i x_i = sum_{i>0} w_i (x_i - x_0) + (sum w_i) x_0
    const int i0 = r.l01 & 0xffffu, i1 = r.l01 >> 16, i2 = r.l23 & 0xffffu, i3 = r.l23 >> 16;
    const float3 e1 = edge(sy, sd, i0, i1), e2 = edge(sy, sd, i0, i2), e3 = edge(sy, sd, i0, i3);
    const float4 w = r.w;
    const float ws = (w.x + w.y) + (w.z + w.w);
    const float4 y0 = sy[i0], d0 = sd[i0];
    const float3 x0 = make_float3(y0.x + d0.x, y0.y + d0.y, y0.z + d0.z);
    const float3 e = make_float3(w.y * e1.x + w.z * e2.x + w.w * e3.x + ws * x0.x,
                                 w.y * e1.y + w.z * e2.y + w.w * e3.y + ws * x0.y,
                                 w.y * e1.z + w.z * e2.z + w.w * e3.z + ws * x0.z);
    const float len = sqrtf(e.x * e.x + e.y * e.y + e.z * e.z);
    float3 p = make_float3(0.f, 0.f, 0.f);
    if (len > 1e-10f && r.nrest > 1e-10f) {
        const float sc = r.nrest / len;
        p = make_float3(e.x * sc, e.y * sc, e.z * sc);
    }
    float3 q;
    if (MODE == kModeConsistent) q = make_float3(r.h2k * (p.x - e.x), r.h2k * (p.y - e.y), r.h2k * (p.z - e.z));
    else                         q = make_float3(r.h2k * p.x, r.h2k * p.y, r.h2k * p.z);
    const int s0 = hbase + e_, s1 = s0 + nhin, s2 = s1 + nhin, s3 = s2 + nhin;
    cx[s0] = w.x * q.x; cy[s0] = w.x * q.y; cz[s0] = w.x * q.z;
    cx[s1] = w.y * q.x; cy[s1] = w.y * q.y; cz[s1] = w.y * q.z;
    cx[s2] = w.z * q.x; cy[s2] = w.z * q.y; cz[s2] = w.z * q.z;
    cx[s3] = w.w * q.x; cy[s3] = w.w * q.y; cz[s3] = w.w * q.z;
}

// Jacobi update of one owned vertex in the consistent form:
// -r = f - m d;  d_hat = d + gamma D^-1 (-r);  d' = omega (d_hat - d_prev) + d_prev.
// Explicit roundings keep every launch structure bitwise identical.
__device__ __forceinline__ float4 update_consistent(float4 d, float4 y, float fx, float fy, float fz, float4 dp,
                                                   float gamma, float omega, float& r2)
{
    const float rx = __fsub_rn(fx, __fmul_rn(y.w, d.x));
    const float ry = __fsub_rn(fy, __fmul_rn(y.w, d.y));
    const float rz = __fsub_rn(fz, __fmul_rn(y.w, d.z));
    float4 o = d;
    if (d.w >= 0.f) {   // free vertex (pinned ones carry -1)
        r2 = __fmaf_rn(rx, rx, __fmaf_rn(ry, ry, __fmul_rn(rz, rz)));
        const float gi = __fmul_rn(gamma, d.w);
        o.x = __fmaf_rn(omega, __fsub_rn(__fmaf_rn(gi, rx, d.x), dp.x), dp.x);
        o.y = __fmaf_rn(omega, __fsub_rn(__fmaf_rn(gi, ry, d.y), dp.y), dp.y);
        o.z = __fmaf_rn(omega, __fsub_rn(__fmaf_rn(gi, rz, d.z), dp.z), dp.z);
    } else {
        r2 = 0.f;
    }
    return o;
}

// x = rhs / diag with rhs = m y + f (src/pd_solver.cu:371-398), stored as x - y.
__device__ __forceinline__ float4 update_literal(float4 d, float4 y, float fx, float fy, float fz)
{
    float4 o = d;
    if (d.w >= 0.f) {
        o.x = __fsub_rn(__fmul_rn(__fmaf_rn(y.w, y.x, fx), d.w), y.x);
        o.y = __fsub_rn(__fmul_rn(__fmaf_rn(y.w, y.y, fy), d.w), y.y);
        o.z = __fsub_rn(__fmul_rn(__fmaf_rn(y.w, y.z, fz), d.w), y.z);
    }
    return o;
}

__device__ __forceinline__ float warp_sum(float v)
{
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ---------------------------------------------------------------------------
// Fused iteration over one patch.  `k` is the sweep index: the block reads
// the offsets d^k = x^k - y from buf[k & 1], reads d^(k-1) and writes d^(k+1)
// in buf[(k+1) & 1] (the same slot, owned by this thread), and accumulates
// ||r(x^k)||^2 into crt[c].acc[k % 3].  With res_only it only evaluates the
// residual.  Data produced by other blocks is loaded with __ldcg (L2, not
// L1), so the same code is correct inside the persistent kernel between
// grid barriers.  Shared memory: sy, sd (float4 per local vertex), then the
// three slot arrays.
// ---------------------------------------------------------------------------
template <int MODE, int NT>
__device__ __forceinline__ void process_patch(const IterArgs& a, const PatchHdr& ph, int k, bool res_only,
                                              float omega, float4* sy, float* cx, float* cy, float* cz,
                                              float* red)
{
    // select, not index: a dynamic index into the parameter struct would
    // copy it to local memory
    const float4* __restrict__ Dk = (k & 1) ? a.buf[1] : a.buf[0];
    float4* __restrict__ Dn = (k & 1) ? a.buf[0] : a.buf[1];
    float4* sd = sy + ph.nlocal;
    const int tid = threadIdx.x;

    // 1. stage y and d^k of owned + halo vertices
    for (int l = tid; l < ph.nlocal; l += NT) {
        const int g = l < ph.nown ? ph.vbegin + l : __ldg(&a.halo[ph.halo_off + l - ph.nown]);
        sy[l] = __ldcg(&a.Y[g]);
        sd[l] = __ldcg(&Dk[g]);
    }
    __syncthreads();

    // 2. local step: triangles then hinges, contributions to shared slots
    const TriRec* __restrict__ tr = a.tris + ph.tri_off;
    const int ntri = ph.ntri, nhin = ph.nhinge;
    for (int t = tid; t < ntri; t += NT) {
        const TriRec r = tr[t];
        triangle_contrib<MODE>(r, sy, sd, t, ntri, cx, cy, cz);
    }
    const HingeRec* __restrict__ hr = a.hinges + ph.hinge_off;
    for (int e = tid; e < nhin; e += NT) {
        const HingeRec r = hr[e];
        hinge_contrib<MODE>(r, sy, sd, e, 3 * ntri, nhin, cx, cy, cz);
    }
    __syncthreads();

    // 3. global step per owned vertex
    const float gamma = a.cinfo[ph.cloth].gamma;
    const int* __restrict__ cp = a.csr_ptr + ph.csr_off;
    const uint16_t* __restrict__ ce = a.csr_ent + ph.ent_off;
    float r2 = 0.f;
    for (int l = tid; l < ph.nown; l += NT) {
        float fx = 0.f, fy = 0.f, fz = 0.f;
        const int b = __ldg(&cp[l]), e = __ldg(&cp[l + 1]);
        for (int q = b; q < e; ++q) {
            const int s = __ldg(&ce[q]);
            fx += cx[s]; fy += cy[s]; fz += cz[s];
        }
        const int g = ph.vbegin + l;
        const float4 d = sd[l];
        const float4 y = sy[l];
        if (MODE == kModeConsistent) {
            float rv;
            const float4 dp = res_only ? d : __ldcg(&Dn[g]);
            const float4 o = update_consistent(d, y, fx, fy, fz, dp, gamma, omega, rv);
            r2 += rv;
            if (!res_only) Dn[g] = o;
        } else if (!res_only) {
            Dn[g] = update_literal(d, y, fx, fy, fz);
        }
    }
    if (MODE == kModeConsistent) {
        r2 = warp_sum(r2);
        if ((tid & 31) == 0) red[tid >> 5] = r2;
        __syncthreads();
        if (tid < 32) {
            float v = tid < NT / 32 ? red[tid] : 0.f;
            v = warp_sum(v);
            if (tid == 0) atomicAdd(&a.crt[ph.cloth].acc[k % 3], (double)v);
        }
    }
}

// Per-cloth decision at the start of sweep k, taken by one thread per block;
// every block of a cloth reaches the same answer from the same data.
// Returns true if the cloth is done.  The cloth's first patch records it.
__device__ __forceinline__ bool cloth_done(const IterArgs& a, int c, int k, bool designated)
{
    ClothRT* rt = a.crt + c;
    if (!__ldcg(&rt->active)) return true;
    const ClothInfo& ci = a.cinfo[c];
    if (k >= 1 && ci.mode == kModeConsistent) {
        const double acc0 = __ldcg(&rt->acc[0]);
        const double rk2 = __ldcg(&rt->acc[(k - 1) % 3]);          // ||r(x^(k-1))||^2
        const double ry2 = (k == 1 && ci.init == 0) ? acc0 : __ldcg(&rt->res_y2);
        if (k == 1 && designated) {
            rt->res0_2 = acc0;
            if (ci.init == 0) rt->res_y2 = acc0;
        }
        if (!isfinite(rk2)) {
            if (designated) { rt->status = -6; rt->used = k - 1; rt->resf_2 = rk2; rt->active = 0; }
            return true;
        }
        if (ci.tol > 0.f && rk2 <= (double)ci.tol * (double)ci.tol * ry2) {
            if (designated) { rt->used = k - 1; rt->resf_2 = rk2; rt->active = 0; }
            return true;
        }
        if (k > ci.max_iter) {   // this cloth's cap: x^max_iter and its residual are final
            if (designated) { rt->used = ci.max_iter; rt->resf_2 = rk2; rt->active = 0; }
            return true;
        }
    }
    if (k >= ci.max_iter && (k > ci.max_iter || !a.have_final)) {
        if (designated) { rt->used = ci.max_iter; rt->resf_2 = -1.0; rt->active = 0; }
        return true;
    }
    return false;
}

__device__ __forceinline__ void reset_rt(ClothRT* crt, int c)
{
    ClothRT r;
    r.active = 1; r.used = 0; r.status = 0; r.warm = 0;
    r.res_y2 = 0.0; r.res0_2 = 0.0; r.resf_2 = -1.0;
    r.acc[0] = r.acc[1] = r.acc[2] = 0.0;
    crt[c] = r;
}

// y = x + h v + h^2 a (w = mass); start iterate into both buffers
// (w = inverse diagonal, -1 for pinned vertices).
__device__ __forceinline__ void predict_vertex(int i, const float4* X, const float4* V, const float4* aux,
                                               const float* mass, const int* vcloth, const ClothInfo* cinfo,
                                               const float4* warm, float4* Y, float4* A, float4* B)
{
    const ClothInfo& ci = cinfo[vcloth[i]];
    const float h = ci.h, h2 = h * h;
    const float4 x = __ldcg(&X[i]), v = __ldcg(&V[i]), au = __ldcg(&aux[i]);
    float4 y;
    y.x = x.x + h * v.x + h2 * ci.ext[0];
    y.y = x.y + h * v.y + h2 * ci.ext[1];
    y.z = x.z + h * v.z + h2 * ci.ext[2];
    y.w = mass[i];
    Y[i] = y;
    // start offset d^0 = x^0 - y
    float4 s;
    if (au.w < 0.f)                    s = make_float4(au.x - y.x, au.y - y.y, au.z - y.z, au.w);  // pin target
    else if (ci.init == 1)             s = make_float4(x.x - y.x, x.y - y.y, x.z - y.z, au.w);     // x_n
    else if (ci.init == 2 && warm) {   const float4 w = __ldcg(&warm[i]); s = make_float4(w.x, w.y, w.z, au.w); }
    else                               s = make_float4(0.f, 0.f, 0.f, au.w);                        // y
    A[i] = s;
    B[i] = s;
}

// Cloths still active after the last sweep keep x^cap.
__device__ __forceinline__ void frame_stats_cloth(const ClothInfo* cinfo, ClothRT* crt, int c, int have_final)
{
    ClothRT* rt = crt + c;
    const ClothInfo& ci = cinfo[c];
    if (ci.max_iter <= 1 && ci.mode == kModeConsistent) {   // the k == 1 bookkeeping never ran
        rt->res0_2 = __ldcg(&rt->acc[0]);
        if (ci.init == 0) rt->res_y2 = rt->res0_2;
    }
    if (__ldcg(&rt->active)) {
        rt->used = ci.max_iter;
        const double rf = __ldcg(&rt->acc[ci.max_iter % 3]);
        rt->resf_2 = (have_final && ci.mode == kModeConsistent) ? rf : -1.0;
        if (have_final && ci.mode == kModeConsistent && !isfinite(rf)) rt->status = -6;
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
    const float h = ci.h, sc = 1.f - ci.damping, ih = 1.f / h;
    V[i] = make_float4(sc * (v.x + h * ci.ext[0] + d.x * ih), sc * (v.y + h * ci.ext[1] + d.y * ih),
                       sc * (v.z + h * ci.ext[2] + d.z * ih), 0.f);
    X[i] = make_float4(y.x + d.x, y.y + d.y, y.z + d.z, 0.f);
}

}  // namespace pdg
