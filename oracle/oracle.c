/*
 * CPU oracle for the PD cloth solve -- TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * This file holds the setup stage (float arithmetic, as the reference does it)
 * and the literal restatement of the reference CUDA step.  The precision-
 * generic solvers live in oracle_solve.inc, included below once for double
 * and once for float.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ======================================================================
 * Generator -- src/mesh_generator.cpp:6-91.
 * Vertex (i, j) at (j*size, 0, i*size); type 0 '\', 1 checkerboard,
 * 2 '/', 3 one centre vertex and four triangles per cell.
 * ====================================================================== */
int orc_grid_counts(int nrows, int ncols, int type, int* N, int* T)
{
    if (nrows < 2 || ncols < 2 || type < 0 || type > 3) return -1;
    const int cells = (nrows - 1) * (ncols - 1);
    *N = nrows * ncols + (type == 3 ? cells : 0);
    *T = cells * (type == 3 ? 4 : 2);
    return 0;
}

void orc_generate_grid(int nrows, int ncols, float size, int type,
                       float* pos, int* tris)
{
    int n = 0;
    for (int i = 0; i < nrows; ++i)
        for (int j = 0; j < ncols; ++j) {
            pos[3 * n + 0] = (float)j * size;
            pos[3 * n + 1] = 0.0f;
            pos[3 * n + 2] = (float)i * size;
            ++n;
        }
    const int cr = nrows - 1, cc = ncols - 1;
    if (type == 3)
        for (int i = 0; i < cr; ++i)
            for (int j = 0; j < cc; ++j) {
                pos[3 * n + 0] = ((float)j + 0.5f) * size;
                pos[3 * n + 1] = 0.0f;
                pos[3 * n + 2] = ((float)i + 0.5f) * size;
                ++n;
            }
    int t = 0;
#define PUT(a, b, c) do { tris[3*t] = (a); tris[3*t+1] = (b); tris[3*t+2] = (c); ++t; } while (0)
    for (int i = 0; i < cr; ++i)
        for (int j = 0; j < cc; ++j) {
            const int v0 = i * ncols + j, v1 = v0 + 1;
            const int v2 = (i + 1) * ncols + j, v3 = v2 + 1;
            if (type == 3) {
                const int c = nrows * ncols + i * cc + j;
                PUT(v0, v1, c); PUT(v1, v3, c); PUT(v3, v2, c); PUT(v2, v0, c);
            } else {
                int back = 1;
                if (type == 1) back = ((i + j) % 2 == 0);
                else if (type == 2) back = 0;
                if (back) { PUT(v0, v1, v3); PUT(v0, v3, v2); }
                else      { PUT(v0, v1, v2); PUT(v1, v3, v2); }
            }
        }
#undef PUT
}

/* ======================================================================
 * Rest state -- src/cloth_mesh.cpp:138-211.
 * P = Gram-Schmidt basis of the rest triangle, Dm = P^T [e1 e2],
 * Dm_inv by the 2x2 cofactor formula, area = |det Dm| / 2,
 * mass += density * area / 3 per corner, dF/dx = kron(Dm_inv^T p, I3).
 * ====================================================================== */
static float norm3f(const float* a) { return sqrtf(a[0]*a[0] + a[1]*a[1] + a[2]*a[2]); }
static float dot3f(const float* a, const float* b) { return a[0]*b[0] + a[1]*b[1] + a[2]*b[2]; }

void orc_rest_state(int N, int T, const float* pos, const int* tris,
                    float density, float* Dm_inv, float* area, float* mass,
                    float* dFdx)
{
    for (int i = 0; i < N; ++i) mass[i] = 0.0f;
    for (int t = 0; t < T; ++t) {
        const int i0 = tris[3*t], i1 = tris[3*t+1], i2 = tris[3*t+2];
        float e1[3], e2[3], P0[3], P1[3], o[3];
        for (int d = 0; d < 3; ++d) {
            e1[d] = pos[3*i1+d] - pos[3*i0+d];
            e2[d] = pos[3*i2+d] - pos[3*i0+d];
        }
        const float n1 = norm3f(e1);
        for (int d = 0; d < 3; ++d) P0[d] = n1 > 0.0f ? e1[d] / n1 : 0.0f;
        const float proj = dot3f(e2, P0);
        for (int d = 0; d < 3; ++d) o[d] = e2[d] - proj * P0[d];
        const float no = norm3f(o);
        if (no > 1e-10f) {
            for (int d = 0; d < 3; ++d) P1[d] = o[d] / no;
        } else {
            float q[3];
            if (fabsf(P0[0]) <= fabsf(P0[1]) && fabsf(P0[0]) <= fabsf(P0[2])) {
                q[0] = 0.0f; q[1] = -P0[2]; q[2] = P0[1];
            } else {
                q[0] = -P0[1]; q[1] = P0[0]; q[2] = 0.0f;
            }
            const float nq = norm3f(q);
            for (int d = 0; d < 3; ++d) P1[d] = nq > 0.0f ? q[d] / nq : 0.0f;
        }
        const float a = dot3f(P0, e1), b = dot3f(P0, e2);
        const float c = dot3f(P1, e1), dd = dot3f(P1, e2);
        const float det = a * dd - c * b;
        const float inv = 1.0f / det;
        const float g00 = dd * inv, g10 = -c * inv, g01 = -b * inv, g11 = a * inv;
        Dm_inv[4*t+0] = g00; Dm_inv[4*t+1] = g10;
        Dm_inv[4*t+2] = g01; Dm_inv[4*t+3] = g11;
        const float A = 0.5f * fabsf(det);
        area[t] = A;
        if (dFdx) {
            /* D = Dm_inv^T * [[-1,1,0],[-1,0,1]] ; row r of D scales I3. */
            const float D[2][3] = {
                { -(g00 + g10), g00, g10 },
                { -(g01 + g11), g01, g11 } };
            float* M = dFdx + 54 * t;
            for (int k = 0; k < 54; ++k) M[k] = 0.0f;
            for (int r = 0; r < 2; ++r)
                for (int v = 0; v < 3; ++v)
                    for (int d = 0; d < 3; ++d)
                        M[(r*3 + d) * 9 + v*3 + d] = D[r][v];
        }
        const float tm = density * A;
        mass[i0] += tm / 3.0f; mass[i1] += tm / 3.0f; mass[i2] += tm / 3.0f;
    }
}

/* ======================================================================
 * Topology -- src/mesh_topology.cpp:11-97.
 * Every triangle edge keyed by (min, max); the first triangle seen is tri_a,
 * the last one tri_b (-1 for a boundary edge).  Edges are returned sorted by
 * key (the reference iterates an unordered_map, whose order is unspecified).
 * ====================================================================== */
typedef struct { int a, b, t, seq; } orc_ekey;
static int cmp_ekey(const void* x, const void* y)
{
    const orc_ekey* p = (const orc_ekey*)x; const orc_ekey* q = (const orc_ekey*)y;
    if (p->a != q->a) return p->a < q->a ? -1 : 1;
    if (p->b != q->b) return p->b < q->b ? -1 : 1;
    return p->seq < q->seq ? -1 : (p->seq > q->seq);
}

int orc_topology(int N, int T, const int* tris, int* edges)
{
    (void)N;
    orc_ekey* k = (orc_ekey*)malloc(sizeof(orc_ekey) * (size_t)(3 * T + 1));
    for (int t = 0; t < T; ++t)
        for (int e = 0; e < 3; ++e) {
            int a = tris[3*t+e], b = tris[3*t+(e+1)%3];
            if (a > b) { const int s = a; a = b; b = s; }
            orc_ekey* q = &k[3*t+e];
            q->a = a; q->b = b; q->t = t; q->seq = 3*t+e;
        }
    qsort(k, (size_t)(3 * T), sizeof(orc_ekey), cmp_ekey);
    int nE = 0;
    for (int i = 0; i < 3 * T;) {
        int j = i;
        while (j + 1 < 3 * T && k[j+1].a == k[i].a && k[j+1].b == k[i].b) ++j;
        edges[4*nE+0] = k[i].a; edges[4*nE+1] = k[i].b;
        edges[4*nE+2] = k[i].t; edges[4*nE+3] = (j > i) ? k[j].t : -1;
        ++nE; i = j + 1;
    }
    free(k);
    return nE;
}

/* ======================================================================
 * Cotangent bend hinges -- src/sim_constraints.cpp:48-127.
 * ====================================================================== */
static int opp_vertex(const int* tris, int t, int v0, int v1)
{
    for (int i = 0; i < 3; ++i) {
        const int v = tris[3*t+i];
        if (v != v0 && v != v1) return v;
    }
    return -1;
}

static float heronf(float a, float b, float c)
{
    const float s = 0.5f * (a + b + c);
    const float v = s * (s - a) * (s - b) * (s - c);
    return v > 0.0f ? sqrtf(v) : 0.0f;
}

static float distf(const float* pos, int i, int j)
{
    float d[3];
    for (int k = 0; k < 3; ++k) d[k] = pos[3*j+k] - pos[3*i+k];
    return norm3f(d);
}

int orc_build_bend(int N, const float* pos, const int* tris, int nE,
                   const int* edges, float kb, int* hinge, float* w,
                   float* n_rest, float* hk)
{
    (void)N;
    int E = 0;
    for (int e = 0; e < nE; ++e) {
        const int v0 = edges[4*e], v1 = edges[4*e+1], ta = edges[4*e+2], tb = edges[4*e+3];
        if (tb == -1) continue;
        const int v2 = opp_vertex(tris, ta, v0, v1), v3 = opp_vertex(tris, tb, v0, v1);
        if (v2 == -1 || v3 == -1) continue;
        const float l01 = distf(pos, v0, v1), l02 = distf(pos, v0, v2), l03 = distf(pos, v0, v3);
        const float l12 = distf(pos, v1, v2), l13 = distf(pos, v1, v3);
        const float A0 = heronf(l01, l02, l12), A1 = heronf(l01, l03, l13);
        if (A0 < 1e-10f || A1 < 1e-10f) continue;
        const float cot02 = (l01*l01 + l12*l12 - l02*l02) / (4.0f * A0);
        const float cot12 = (l01*l01 + l02*l02 - l12*l12) / (4.0f * A0);
        const float cot03 = (l01*l01 + l13*l13 - l03*l03) / (4.0f * A1);
        const float cot13 = (l01*l01 + l03*l03 - l13*l13) / (4.0f * A1);
        const float w0 = cot02 + cot03, w1 = cot12 + cot13;
        const float w2 = -(cot02 + cot12), w3 = -(cot03 + cot13);
        float er[3];
        for (int d = 0; d < 3; ++d)
            er[d] = w0*pos[3*v0+d] + w1*pos[3*v1+d] + w2*pos[3*v2+d] + w3*pos[3*v3+d];
        hinge[4*E+0] = v0; hinge[4*E+1] = v1; hinge[4*E+2] = v2; hinge[4*E+3] = v3;
        w[4*E+0] = w0; w[4*E+1] = w1; w[4*E+2] = w2; w[4*E+3] = w3;
        n_rest[E] = norm3f(er);
        hk[E] = kb;
        ++E;
    }
    return E;
}

/* Jacobi diagonal -- src/sim_constraints.cpp:133-192. */
void orc_jacobi_diag(int N, int T, const int* tris, const float* Dm_inv,
                     const float* area, const float* k_stretch, int E,
                     const int* hinge, const float* w, const float* hk,
                     const float* mass, float h, float* diag)
{
    const float h2 = h * h;
    for (int i = 0; i < N; ++i) diag[i] = mass[i];
    for (int t = 0; t < T; ++t) {
        const float wA = k_stretch[t] * area[t];
        const float g00 = Dm_inv[4*t], g10 = Dm_inv[4*t+1], g01 = Dm_inv[4*t+2], g11 = Dm_inv[4*t+3];
        const float s0 = g00 + g10, s1 = g01 + g11;
        diag[tris[3*t+0]] += h2 * wA * (s0*s0 + s1*s1);
        diag[tris[3*t+1]] += h2 * wA * (g00*g00 + g01*g01);
        diag[tris[3*t+2]] += h2 * wA * (g10*g10 + g11*g11);
    }
    for (int e = 0; e < E; ++e)
        for (int i = 0; i < 4; ++i) {
            const float wi = w[4*e+i];
            diag[hinge[4*e+i]] += h2 * hk[e] * wi * wi;
        }
}

/* ======================================================================
 * Literal step -- src/pd_solver.cu:496-621 with the kernels at :18-428.
 * Reproduces the reference's update x <- rhs / diag (no off-diagonal
 * subtraction), its eigenvector-based 2x2 rotation (which is the transpose
 * of the polar rotation), and its pin handling.  rhs is summed in a fixed
 * order where the GPU uses atomics.
 * ====================================================================== */
static void literal_project(const float* x, const int* tri, const float* G, float R[6])
{
    const float* p0 = x + 3*tri[0]; const float* p1 = x + 3*tri[1]; const float* p2 = x + 3*tri[2];
    float ds0[3], ds1[3], F0[3], F1[3], u1[3], u2[3];
    for (int d = 0; d < 3; ++d) { ds0[d] = p1[d] - p0[d]; ds1[d] = p2[d] - p0[d]; }
    const float m00 = G[0], m10 = G[1], m01 = G[2], m11 = G[3];
    for (int d = 0; d < 3; ++d) {
        F0[d] = ds0[d]*m00 + ds1[d]*m10;
        F1[d] = ds0[d]*m01 + ds1[d]*m11;
    }
    const float lf0 = norm3f(F0);
    if (lf0 > 1e-10f) { for (int d = 0; d < 3; ++d) u1[d] = F0[d] / lf0; }
    else { u1[0] = 1.0f; u1[1] = 0.0f; u1[2] = 0.0f; }
    const float f1u1 = dot3f(F1, u1);
    float up[3];
    for (int d = 0; d < 3; ++d) up[d] = F1[d] - f1u1 * u1[d];
    const float lup = norm3f(up);
    if (lup > 1e-10f) { for (int d = 0; d < 3; ++d) u2[d] = up[d] / lup; }
    else {
        if (fabsf(u1[0]) > 0.9f) { u2[0] = -u1[1]; u2[1] = u1[0]; u2[2] = 0.0f; }
        else { u2[0] = 0.0f; u2[1] = -u1[2]; u2[2] = u1[1]; }
        const float l = norm3f(u2);
        for (int d = 0; d < 3; ++d) u2[d] /= l;
    }
    const float F00 = dot3f(u1, F0), F01 = dot3f(u1, F1), F10 = dot3f(u2, F0), F11 = dot3f(u2, F1);
    const float A00 = F00*F00 + F10*F10, A01 = F00*F01 + F10*F11, A11 = F01*F01 + F11*F11;
    const float tr = (A00 + A11) * 0.5f;
    const float disc = sqrtf(fmaxf(0.0f, (A00 - A11)*(A00 - A11)*0.25f + A01*A01));
    const float l1 = tr + disc, l2 = tr - disc;
    float v1x, v1y, v2x, v2y;
    if (disc < 1e-10f || fabsf(A01) < 1e-10f) { v1x = 1.0f; v1y = 0.0f; v2x = 0.0f; v2y = 1.0f; }
    else {
        const float tmp = l1 - A00;
        const float len = sqrtf(A01*A01 + tmp*tmp);
        if (len > 1e-10f) { v1x = A01 / len; v1y = tmp / len; } else { v1x = 1.0f; v1y = 0.0f; }
        v2x = -v1y; v2y = v1x;
    }
    const float s1 = sqrtf(fmaxf(0.0f, l1)), s2 = sqrtf(fmaxf(0.0f, l2));
    float w1x, w1y, w2x, w2y;
    if (s1 > 1e-10f) { w1x = (F00*v1x + F01*v1y) / s1; w1y = (F10*v1x + F11*v1y) / s1; }
    else { w1x = 1.0f; w1y = 0.0f; }
    if (s2 > 1e-10f) { w2x = (F00*v2x + F01*v2y) / s2; w2y = (F10*v2x + F11*v2y) / s2; }
    else {
        const float fx = F00*v2x + F01*v2y, fy = F10*v2x + F11*v2y;
        const float dd = w1x*fx + w1y*fy;
        const float wx = fx - dd*w1x, wy = fy - dd*w1y;
        const float l = sqrtf(wx*wx + wy*wy);
        if (l > 1e-10f) { w2x = wx / l; w2y = wy / l; } else { w2x = -w1y; w2y = w1x; }
    }
    const float r00 = v1x*w1x + v2x*w2x, r01 = v1x*w1y + v2x*w2y;
    const float r10 = v1y*w1x + v2y*w2x, r11 = v1y*w1y + v2y*w2y;
    for (int d = 0; d < 3; ++d) {
        R[d]     = u1[d]*r00 + u2[d]*r10;
        R[3 + d] = u1[d]*r01 + u2[d]*r11;
    }
}

void orc_step_literal_f32(const orc_problem* p, const float* diag, int iters,
                          float* x, float* v)
{
    const int N = p->N;
    const float h = (float)p->h, h2 = h * h;
    float* y    = (float*)malloc(sizeof(float) * 3 * N);
    float* xp   = (float*)malloc(sizeof(float) * 3 * N);
    float* xo   = (float*)malloc(sizeof(float) * 3 * N);
    float* rhs  = (float*)malloc(sizeof(float) * 3 * N);
    float* R    = (float*)malloc(sizeof(float) * 6 * (p->T > 0 ? p->T : 1));
    float* bp   = (float*)malloc(sizeof(float) * 3 * (p->E > 0 ? p->E : 1));
    memcpy(xp, x, sizeof(float) * 3 * N);
    const float e0 = (float)p->ext[0], e1 = (float)p->ext[1], e2 = (float)p->ext[2];
    for (int i = 0; i < N; ++i) {
        /* predict_kernel: gravity enters as dt*dt*g on y only; the external
         * x/z terms extend it for wind (zero in the reference). */
        y[3*i+0] = x[3*i+0] + h * v[3*i+0] + h2 * e0;
        y[3*i+1] = x[3*i+1] + h * v[3*i+1] + h2 * e1;
        y[3*i+2] = x[3*i+2] + h * v[3*i+2] + h2 * e2;
    }
    float* xin = x;
    float* xout = xo;
    for (int it = 0; it < iters; ++it) {
        for (int t = 0; t < p->T; ++t) literal_project(xin, p->tris + 3*t, p->Dm_inv + 4*t, R + 6*t);
        for (int e = 0; e < p->E; ++e) {
            float acc[3] = {0.0f, 0.0f, 0.0f};
            for (int i = 0; i < 4; ++i) {
                const int vi = p->hinge[4*e+i]; const float wi = p->hinge_w[4*e+i];
                for (int d = 0; d < 3; ++d) acc[d] += wi * xin[3*vi+d];
            }
            const float nr = p->hinge_n[e];
            const float len = norm3f(acc);
            for (int d = 0; d < 3; ++d)
                bp[3*e+d] = (len > 1e-10f && nr > 1e-10f) ? acc[d] * (nr / len) : 0.0f;
        }
        for (int i = 0; i < 3 * N; ++i) rhs[i] = 0.0f;
        for (int t = 0; t < p->T; ++t) {
            const int* tv = p->tris + 3*t; const float* G = p->Dm_inv + 4*t; const float* Rt = R + 6*t;
            const float g00 = G[0], g10 = G[1], g01 = G[2], g11 = G[3];
            const float wA = p->k_stretch[t] * p->area[t] * h2;
            for (int d = 0; d < 3; ++d) {
                rhs[3*tv[0]+d] += -((g00+g10)*Rt[d] + (g01+g11)*Rt[3+d]) * wA;
                rhs[3*tv[1]+d] += (g00*Rt[d] + g01*Rt[3+d]) * wA;
                rhs[3*tv[2]+d] += (g10*Rt[d] + g11*Rt[3+d]) * wA;
            }
        }
        for (int e = 0; e < p->E; ++e) {
            const float k = p->hinge_k[e] * h2;
            for (int i = 0; i < 4; ++i) {
                const int vi = p->hinge[4*e+i]; const float wi = p->hinge_w[4*e+i];
                for (int d = 0; d < 3; ++d) rhs[3*vi+d] += k * wi * bp[3*e+d];
            }
        }
        for (int i = 0; i < N; ++i)
            for (int d = 0; d < 3; ++d) rhs[3*i+d] += p->mass[i] * y[3*i+d];
        for (int i = 0; i < N; ++i) {
            const float dg = diag[i];
            const float inv = dg > 1e-10f ? 1.0f / dg : 0.0f;
            for (int d = 0; d < 3; ++d) xout[3*i+d] = rhs[3*i+d] * inv;
        }
        for (int q = 0; q < p->P; ++q) {
            const int idx = p->pin_idx[q];
            for (int d = 0; d < 3; ++d) { xout[3*idx+d] = p->pin_target[3*q+d]; v[3*idx+d] = 0.0f; }
        }
        float* s = xin; xin = xout; xout = s;
    }
    if (xin != x) memcpy(x, xin, sizeof(float) * 3 * N);
    const float sc = (1.0f - (float)p->damping) / h;
    for (int i = 0; i < 3 * N; ++i) v[i] = (x[i] - xp[i]) * sc;
    for (int q = 0; q < p->P; ++q) {
        const int idx = p->pin_idx[q];
        for (int d = 0; d < 3; ++d) { x[3*idx+d] = p->pin_target[3*q+d]; v[3*idx+d] = 0.0f; }
    }
    free(y); free(xp); free(xo); free(rhs); free(R); free(bp);
}

/* ---------------- precision-generic solvers ---------------- */
/* size of the last LDL^T factor the direct solve built (strictly lower
 * entries of L), for the CPU-baseline report */
static long long orc_last_nnz_L = 0;
long long orc_last_factor_nnz(void) { return orc_last_nnz_L; }

#define REAL double
#define SFX(name) name##_f64
#define RSQRT(a) sqrt(a)
#define RFABS(a) fabs(a)
#include "oracle_solve.inc"
#undef REAL
#undef SFX
#undef RSQRT
#undef RFABS

#define REAL float
#define SFX(name) name##_f32
#define RSQRT(a) sqrtf(a)
#define RFABS(a) fabsf(a)
#define ORC_SECOND_PASS 1
#include "oracle_solve.inc"
#undef REAL
#undef SFX
#undef RSQRT
#undef RFABS
