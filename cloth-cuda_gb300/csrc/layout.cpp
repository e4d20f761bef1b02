// Host-side construction of the device layout: every cloth reordered so that
// its patches are compact tiles (recursive coordinate bisection, Z-order
// inside a tile), cut into patches, local triangle/hinge records with 16-bit
// vertex references, and per-vertex gather lists (CSR) over contribution
// slots.
#include "pdg_solver.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>

namespace pdg {

namespace {

// A record that fills a gap before a group boundary: never read by a kernel
// (they read records c < ncell of their patch); no outputs.
CellRec pad_cell()
{
    CellRec r{};
    r.vm01 = r.vm23 = r.vm45 = 0xffffffffu;
    return r;
}

uint32_t spread10(uint32_t v)
{
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

// Vertex order along the Z-order curve of the rest positions (one cube
// spanning the bounding box, 10 bits per axis); ties keep input order.
void morton_order(const MeshData& m, std::vector<int>& perm)
{
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = 0; i < m.N; ++i)
        for (int d = 0; d < 3; ++d) {
            lo[d] = std::min(lo[d], m.rest[3 * i + d]);
            hi[d] = std::max(hi[d], m.rest[3 * i + d]);
        }
    float ext = 0.f;
    for (int d = 0; d < 3; ++d) ext = std::max(ext, hi[d] - lo[d]);
    const float sc = ext > 0.f ? 1023.f / ext : 0.f;
    std::vector<uint64_t> key(m.N);
    for (int i = 0; i < m.N; ++i) {
        uint32_t q[3];
        for (int d = 0; d < 3; ++d) {
            const float f = (m.rest[3 * i + d] - lo[d]) * sc;
            q[d] = (uint32_t)std::min(1023.f, std::max(0.f, f));
        }
        const uint32_t code = spread10(q[0]) | (spread10(q[1]) << 1) | (spread10(q[2]) << 2);
        key[i] = ((uint64_t)code << 32) | (uint32_t)i;
    }
    std::sort(key.begin(), key.end());
    perm.resize(m.N);
    for (int i = 0; i < m.N; ++i) perm[i] = (int)(key[i] & 0xffffffffu);
}

// Vertex order whose consecutive runs of `pv` vertices are compact regions of
// the rest shape: recursive coordinate bisection.  A range holding np
// patches is split across its bounding box's longest axis so that the lower
// part holds floor(np/2) whole patches; a range of one patch keeps the
// Z-order curve inside (ties by vertex index, so the order is deterministic).
void bisection_order(const MeshData& m, int pv, std::vector<int>& perm)
{
    std::vector<int> z;
    morton_order(m, z);
    std::vector<int> zrank(m.N);
    for (int i = 0; i < m.N; ++i) zrank[z[i]] = i;
    perm = z;
    struct Range { int b, e; };
    std::vector<Range> stack{{0, m.N}};
    while (!stack.empty()) {
        const Range r = stack.back();
        stack.pop_back();
        const int n = r.e - r.b;
        const int np = (n + pv - 1) / pv;
        if (np <= 1) {
            std::sort(perm.begin() + r.b, perm.begin() + r.e, [&](int a, int b) { return zrank[a] < zrank[b]; });
            continue;
        }
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int i = r.b; i < r.e; ++i)
            for (int d = 0; d < 3; ++d) {
                lo[d] = std::min(lo[d], m.rest[3 * perm[i] + d]);
                hi[d] = std::max(hi[d], m.rest[3 * perm[i] + d]);
            }
        int ax = 0;
        for (int d = 1; d < 3; ++d)
            if (hi[d] - lo[d] > hi[ax] - lo[ax]) ax = d;
        const int mid = r.b + (np / 2) * pv;
        std::nth_element(perm.begin() + r.b, perm.begin() + mid, perm.begin() + r.e, [&](int a, int b) {
            const float fa = m.rest[3 * a + ax], fb = m.rest[3 * b + ax];
            return fa < fb || (fa == fb && a < b);
        });
        stack.push_back({r.b, mid});
        stack.push_back({mid, r.e});
    }
}

// Dm_inv of a triangle whose corners are rotated by r places, (p0, p1, p2)
// -> (p_r, p_r+1, p_r+2).  Rows of G weight the two edge vectors (F = Ds G,
// row 0 with x1 - x0, row 1 with x2 - x0); one rotation maps the edges to
// (e2 - e1, -e1), so the rows become (row1, -(row0 + row1)).
float4 rotate_G(const float* G, int r)
{
    float a0 = G[0], a1 = G[2], b0 = G[1], b1 = G[3];   // row 0 = (g00, g01), row 1 = (g10, g11)
    for (int q = 0; q < r; ++q) {
        const float n0 = -(a0 + b0), n1 = -(a1 + b1);
        a0 = b0; a1 = b1;
        b0 = n0; b1 = n1;
    }
    return make_float4(a0, b0, a1, b1);
}

// A cell of one cloth in cloth vertex ids, with its record payload; the
// local indices and slots are filled in per patch.
struct CellBuild {
    int v[6];        // c0, c1, c2, c3, x1, x2 (-1: absent)
    CellRec rec;
};

// The cells of one cloth, independent of the patch cut, so every patch size
// and launch structure sums the same contributions in the same order.
//  1. Triangles are paired across shared edges, longest edge first (the
//     diagonals of a grid's quads), greedily; a pair must be consistently
//     oriented and have distinct apexes.
//  2. One cell per pair, numbered by its lower triangle, and one per
//     unpaired triangle.  The hinge of a pair's shared edge is its h0.
//  3. Every other hinge lies on an edge between two cells and goes to one of
//     them as h1 / h2 (at most two per cell): greedily to the less loaded
//     one, else along an augmenting path of moves.  What is left over stays
//     a lone hinge.
void build_cells(const MeshData& m, const Topology& tp, const ConstraintData& cd, float h2,
                 std::vector<CellBuild>& cells, std::vector<int>& lone)
{
    const int T = m.T, E = (int)cd.bend_k.size();
    const int nedge = (int)(tp.edges.size() / 4);
    auto tv = [&](int t, int k) { return m.tris[3 * t + (k % 3)]; };
    // corner k of triangle t such that (p_k, p_k+1) = (a, b), else -1
    auto side = [&](int t, int a, int b) {
        for (int k = 0; k < 3; ++k)
            if (tv(t, k) == a && tv(t, k + 1) == b) return k;
        return -1;
    };
    auto apex = [&](int t, int a, int b) {
        for (int k = 0; k < 3; ++k)
            if (tv(t, k) != a && tv(t, k) != b) return tv(t, k);
        return -1;
    };
    // topology edge of the vertex pair (a, b), -1 if none (edges are sorted)
    auto find_edge = [&](int a, int b) {
        if (a > b) std::swap(a, b);
        int lo = 0, hi = nedge;
        while (lo < hi) {
            const int mid = (lo + hi) / 2;
            const int u = tp.edges[4 * mid], w = tp.edges[4 * mid + 1];
            if (u < a || (u == a && w < b)) lo = mid + 1; else hi = mid;
        }
        return (lo < nedge && tp.edges[4 * lo] == a && tp.edges[4 * lo + 1] == b) ? lo : -1;
    };

    // 1. pairing
    std::vector<int> cand;
    for (int e = 0; e < nedge; ++e) {
        const int v0 = tp.edges[4 * e], v1 = tp.edges[4 * e + 1], ta = tp.edges[4 * e + 2], tb = tp.edges[4 * e + 3];
        if (tb < 0 || ta == tb) continue;
        const bool fwd = side(ta, v0, v1) >= 0;
        if (!(fwd ? side(tb, v1, v0) >= 0 : (side(ta, v1, v0) >= 0 && side(tb, v0, v1) >= 0))) continue;
        if (apex(ta, v0, v1) == apex(tb, v0, v1)) continue;
        cand.push_back(e);
    }
    std::stable_sort(cand.begin(), cand.end(), [&](int p, int q) { return tp.rest_len[p] > tp.rest_len[q]; });
    std::vector<int> partner(T, -1), pedge(T, -1);
    for (int e : cand) {
        const int ta = tp.edges[4 * e + 2], tb = tp.edges[4 * e + 3];
        if (partner[ta] >= 0 || partner[tb] >= 0) continue;
        partner[ta] = tb; partner[tb] = ta;
        pedge[ta] = pedge[tb] = e;
    }

    // 2. cells
    cells.clear();
    std::vector<int> cell_of(T, -1);
    auto stretch = [&](int t) { return h2 * ((t < (int)cd.k_stretch.size() ? cd.k_stretch[t] : 0.f) * m.area[t]); };
    for (int t = 0; t < T; ++t) {
        if (partner[t] >= 0 && partner[t] < t) continue;
        CellBuild c{};
        for (int& x : c.v) x = -1;
        const int u = partner[t];
        int r0 = 0;
        if (u >= 0) {
            const int a = tp.edges[4 * pedge[t]], b = tp.edges[4 * pedge[t] + 1];
            r0 = side(t, a, b);
            if (r0 < 0) r0 = side(t, b, a);
        }
        c.v[0] = tv(t, r0); c.v[1] = tv(t, r0 + 1); c.v[2] = tv(t, r0 + 2);
        c.rec.G0 = rotate_G(&m.Dm_inv[4 * t], r0);
        c.rec.h2wA0 = stretch(t);
        if (u >= 0) {
            const int r1 = side(u, c.v[1], c.v[0]);
            c.v[3] = tv(u, r1 + 2);
            c.rec.G1 = rotate_G(&m.Dm_inv[4 * u], r1);
            c.rec.h2wA1 = stretch(u);
            cell_of[u] = (int)cells.size();
        }
        cell_of[t] = (int)cells.size();
        cells.push_back(c);
    }
    const int C = (int)cells.size();

    // weights of hinge e over c0..c3 and its corner outside the cell (-1: none)
    auto cell_weights = [&](const CellBuild& c, int e, float4& W, float& wx) {
        float w[4] = {0.f, 0.f, 0.f, 0.f};
        int x = -1;
        wx = 0.f;
        for (int j = 0; j < 4; ++j) {
            const int v = cd.quads[4 * e + j];
            int k = 0;
            while (k < 4 && c.v[k] != v) ++k;
            if (k < 4) w[k] = cd.w[4 * e + j];
            else { x = v; wx = cd.w[4 * e + j]; }
        }
        W = make_float4(w[0], w[1], w[2], w[3]);
        return x;
    };

    // 3. hinges: h0 of a pair, else an outer hinge of one of its two cells
    std::vector<int> h0(C, -1);
    std::vector<std::array<int, 2>> ca(E, {-1, -1});   // candidate cells
    lone.clear();
    for (int e = 0; e < E; ++e) {
        const int* q = &cd.quads[4 * e];
        const int te = find_edge(q[0], q[1]);
        int c0 = -1, c1 = -1;
        if (te >= 0 && tp.edges[4 * te + 3] >= 0) {
            const int ta = tp.edges[4 * te + 2], tb = tp.edges[4 * te + 3];
            const int pa = apex(ta, q[0], q[1]), pb = apex(tb, q[0], q[1]);
            if ((pa == q[2] && pb == q[3]) || (pa == q[3] && pb == q[2])) { c0 = cell_of[ta]; c1 = cell_of[tb]; }
        }
        if (c0 < 0) { lone.push_back(e); continue; }
        if (c0 == c1) {
            if (h0[c0] < 0) h0[c0] = e; else lone.push_back(e);
            continue;
        }
        ca[e] = {c0, c1};
    }
    std::vector<std::array<int, 2>> held(C, {-1, -1});
    auto nheld = [&](int c) { return (held[c][0] >= 0) + (held[c][1] >= 0); };
    auto put = [&](int c, int e) { held[c][held[c][0] >= 0 ? 1 : 0] = e; };
    auto take = [&](int c, int e) { held[c][held[c][0] == e ? 0 : 1] = -1; };
    std::vector<int> from_c(C, -1), from_h(C, -1), seen(C, -1), queue;
    for (int e = 0; e < E; ++e) {
        if (ca[e][0] < 0) continue;
        const int a = ca[e][0], b = ca[e][1];
        const int best = nheld(b) < nheld(a) ? b : a;
        if (nheld(best) < 2) { put(best, e); continue; }
        // augmenting path: move held hinges to their other cell until one
        // has room (breadth first, bounded)
        queue.clear();
        for (int c : {a, b}) { seen[c] = e; from_c[c] = -1; from_h[c] = e; queue.push_back(c); }
        int found = -1;
        for (size_t qi = 0; qi < queue.size() && found < 0 && queue.size() < 512; ++qi) {
            const int c = queue[qi];
            for (int s2 = 0; s2 < 2 && found < 0; ++s2) {
                const int f = held[c][s2];
                if (f < 0) continue;
                const int o = ca[f][0] == c ? ca[f][1] : ca[f][0];
                if (seen[o] == e) continue;
                seen[o] = e; from_c[o] = c; from_h[o] = f;
                if (nheld(o) < 2) found = o; else queue.push_back(o);
            }
        }
        if (found < 0) { lone.push_back(e); continue; }
        for (int c = found; c >= 0;) {   // c gains from_h[c], which leaves from_c[c]
            const int f = from_h[c], p = from_c[c];
            if (p >= 0) take(p, f);
            put(c, f);
            c = p;
        }
    }
    std::sort(lone.begin(), lone.end());

    // 4. hinge payloads, outer hinges in hinge order
    for (int c = 0; c < C; ++c) {
        CellBuild& cb = cells[c];
        CellRec& r = cb.rec;
        if (h0[c] >= 0) {
            float wx;
            cell_weights(cb, h0[c], r.W0, wx);
            r.h2k0 = h2 * cd.bend_k[h0[c]];
            r.nrest0 = cd.n_rest[h0[c]];
        }
        std::array<int, 2> hs = held[c];
        if (hs[0] < 0 || (hs[1] >= 0 && hs[1] < hs[0])) std::swap(hs[0], hs[1]);
        for (int j = 0; j < 2; ++j) {
            const int e = hs[j];
            if (e < 0) continue;
            float4 W;
            float wx;
            const int x = cell_weights(cb, e, W, wx);
            (j == 0 ? r.W1 : r.W2) = W;
            (j == 0 ? r.wx1 : r.wx2) = wx;
            (j == 0 ? r.h2k1 : r.h2k2) = h2 * cd.bend_k[e];
            (j == 0 ? r.nrest1 : r.nrest2) = cd.n_rest[e];
            cb.v[4 + j] = x;
        }
    }
}

}  // namespace

bool build_layout(const std::vector<ClothSetup>& cl, int patch_verts, HostLayout& L, std::string& err)
{
    L = HostLayout();
    const int C = (int)cl.size();
    L.ncloth = C;
    int ntot = 0;
    for (const auto& c : cl) ntot += c.mesh->N;
    L.ntot = ntot;
    L.perm_global.resize(ntot);
    L.perm_local.resize(ntot);
    L.vcloth.resize(ntot);
    L.mass.resize(ntot);
    L.aux.resize(ntot);
    L.cinfo.resize(C);
    L.cap = 0;
    for (const auto& c : cl) L.cap = std::max(L.cap, c.cfg.max_iterations);
    L.omega.assign((size_t)C * std::max(1, L.cap), 1.f);
    L.omega_stride = std::max(1, L.cap);

    int vbase = 0;
    for (int ci = 0; ci < C; ++ci) {
        const MeshData& m = *cl[ci].mesh;
        const Topology& tp = *cl[ci].topo;
        const ConstraintData& cd = cl[ci].cons;
        const pdg_config& cfg = cl[ci].cfg;
        const int N = m.N;
        std::vector<int> perm, iperm(N);
        bisection_order(m, patch_verts, perm);
        for (int i = 0; i < N; ++i) iperm[perm[i]] = i;
        const float h2 = cfg.dt * cfg.dt;
        std::vector<CellBuild> cells;
        std::vector<int> lone;
        build_cells(m, tp, cd, h2, cells, lone);
        const int C = (int)cells.size(), H = (int)lone.size();
        // A vertex is "boundary" when a cell or lone hinge through it has a
        // corner in another patch (it is then in that patch's halo).  Within
        // each patch the boundary vertices go first, so a kernel can finish
        // and publish them before the interior.
        std::vector<char> bnd(N, 0);
        {
            auto mark = [&](const int* v, int n) {
                int p = -1;
                bool span = false;
                for (int a = 0; a < n; ++a) {
                    if (v[a] < 0) continue;
                    const int q = iperm[v[a]] / patch_verts;
                    span = span || (p >= 0 && q != p);
                    p = q;
                }
                if (span)
                    for (int a = 0; a < n; ++a)
                        if (v[a] >= 0) bnd[v[a]] = 1;
            };
            for (int c = 0; c < C; ++c) mark(cells[c].v, 6);
            for (int e : lone) mark(&cd.quads[4 * e], 4);
            for (int p0 = 0; p0 < N; p0 += patch_verts)
                std::stable_partition(perm.begin() + p0, perm.begin() + std::min(N, p0 + patch_verts),
                                      [&](int o) { return bnd[o] != 0; });
            for (int i = 0; i < N; ++i) iperm[perm[i]] = i;
        }

        std::vector<float> diag;
        jacobi_diag(m, cd, cfg.dt, diag);
        std::vector<int> pin_slot(N, -1);
        for (size_t q = 0; q < cd.pins.size(); ++q) pin_slot[cd.pins[q]] = (int)q;
        for (int i = 0; i < N; ++i) {
            const int o = perm[i], g = vbase + i;
            L.perm_global[g] = vbase + o;
            L.perm_local[g] = o;
            L.vcloth[g] = ci;
            L.mass[g] = m.mass[o];
            const float dg = diag[o];
            if (pin_slot[o] >= 0) {
                const int q = pin_slot[o];
                L.aux[g] = make_float4(cd.targets[3 * q], cd.targets[3 * q + 1], cd.targets[3 * q + 2], -1.f);
            } else {
                L.aux[g] = make_float4(0.f, 0.f, 0.f, dg > 1e-10f ? 1.0f / dg : 0.f);
            }
        }

        ClothInfo info{};
        info.vbegin = vbase;
        info.nverts = N;
        info.patch_begin = (int)L.patches.size();
        info.max_iter = cfg.max_iterations;
        info.use_cheb = cfg.use_chebyshev;
        info.cheb_delay = cfg.cheb_delay;
        info.mode = cfg.mode;
        info.init = cfg.mode == PDG_MODE_REFERENCE_LITERAL ? PDG_INIT_PREVIOUS : cfg.init;
        info.h = cfg.dt;
        info.damping = cfg.damping;
        info.gamma = cfg.gamma;
        info.tol = cfg.mode == PDG_MODE_REFERENCE_LITERAL ? 0.f : cfg.tolerance;
        info.rho = cfg.rho;
        info.ext[0] = cfg.wind[0];
        info.ext[1] = cfg.gravity + cfg.wind[1];
        info.ext[2] = cfg.wind[2];
        // Chebyshev weights omega_k of sweep k (DESIGN of the reference,
        // omega_1 = 1, omega_2 = 2/(2 - rho^2), omega_k+1 = 4/(4 - rho^2 omega_k))
        {
            float om = 1.f;
            const float r2 = cfg.rho * cfg.rho;
            for (int k = 0; k < cfg.max_iterations; ++k) {
                if (!cfg.use_chebyshev || cfg.mode == PDG_MODE_REFERENCE_LITERAL || k < cfg.cheb_delay) om = 1.f;
                else if (k == cfg.cheb_delay) om = 2.f / (2.f - r2);
                else om = 4.f / (4.f - r2 * om);
                L.omega[(size_t)ci * L.omega_stride + k] = om;
            }
        }

        // vertex -> cell and vertex -> lone hinge lists
        std::vector<int> vc_ptr(N + 1, 0), vc, vh_ptr(N + 1, 0), vh;
        {
            for (int c = 0; c < C; ++c)
                for (int k = 0; k < 6; ++k)
                    if (cells[c].v[k] >= 0) vc_ptr[cells[c].v[k] + 1]++;
            for (int q = 0; q < H; ++q)
                for (int a = 0; a < 4; ++a) vh_ptr[cd.quads[4 * lone[q] + a] + 1]++;
            for (int i = 0; i < N; ++i) { vc_ptr[i + 1] += vc_ptr[i]; vh_ptr[i + 1] += vh_ptr[i]; }
            vc.resize(vc_ptr[N]);
            vh.resize(vh_ptr[N]);
            std::vector<int> f(vc_ptr.begin(), vc_ptr.end() - 1), g(vh_ptr.begin(), vh_ptr.end() - 1);
            for (int c = 0; c < C; ++c)
                for (int k = 0; k < 6; ++k)
                    if (cells[c].v[k] >= 0) vc[f[cells[c].v[k]]++] = c;
            for (int q = 0; q < H; ++q)
                for (int a = 0; a < 4; ++a) vh[g[cd.quads[4 * lone[q] + a]]++] = q;
        }

        std::vector<int> cmark(C, -1), hmark(H, -1), vmark(N, -1), vloc(N, 0);
        std::vector<int> lcell, lhin, halo, cnt;
        for (int p0 = 0; p0 < N; p0 += patch_verts) {
            const int p1 = std::min(N, p0 + patch_verts);
            const int nown = p1 - p0;
            const int stamp = (int)L.patches.size();
            lcell.clear(); lhin.clear(); halo.clear();
            int nbnd_p = 0, ncell_a = 0, nhin_a = 0;
            for (int l = 0; l < nown; ++l) {
                const int o = perm[p0 + l];
                for (int q = vc_ptr[o]; q < vc_ptr[o + 1]; ++q) {
                    const int c = vc[q];
                    if (cmark[c] != stamp) { cmark[c] = stamp; lcell.push_back(c); }
                }
                for (int q = vh_ptr[o]; q < vh_ptr[o + 1]; ++q) {
                    const int e = vh[q];
                    if (hmark[e] != stamp) { hmark[e] = stamp; lhin.push_back(e); }
                }
            }
            std::sort(lcell.begin(), lcell.end());
            std::sort(lhin.begin(), lhin.end());
            auto touch = [&](int o) {
                if (o < 0) return;
                const int n = iperm[o];
                if (n >= p0 && n < p1) return;
                if (vmark[n] != stamp) { vmark[n] = stamp; halo.push_back(n); }
            };
            for (int c : lcell)
                for (int k = 0; k < 6; ++k) touch(cells[c].v[k]);
            for (int q : lhin)
                for (int a = 0; a < 4; ++a) touch(cd.quads[4 * lone[q] + a]);
            std::sort(halo.begin(), halo.end());
            for (int l = 0; l < nown; ++l) vloc[p0 + l] = l;
            for (size_t q = 0; q < halo.size(); ++q) vloc[halo[q]] = nown + (int)q;
            auto loc = [&](int o) { return (uint32_t)vloc[iperm[o]]; };
            // record placement follows the vertex order of the lowest local
            // corner, so the lanes of a warp touch neighbouring vertices and
            // neighbouring slots (fewer shared-memory bank conflicts); the
            // summation order is fixed separately below
            {
                auto lo_c = [&](int c) {
                    int lo = 1 << 30;
                    for (int k = 0; k < 6; ++k)
                        if (cells[c].v[k] >= 0) lo = std::min(lo, (int)loc(cells[c].v[k]));
                    return lo;
                };
                auto lo_h = [&](int q) {
                    int lo = (int)loc(cd.quads[4 * lone[q]]);
                    for (int a = 1; a < 4; ++a) lo = std::min(lo, (int)loc(cd.quads[4 * lone[q] + a]));
                    return lo;
                };
                std::stable_sort(lcell.begin(), lcell.end(), [&](int u, int w) { return lo_c(u) < lo_c(w); });
                std::stable_sort(lhin.begin(), lhin.end(), [&](int u, int w) { return lo_h(u) < lo_h(w); });
                // boundary vertices are local 0..nbnd-1; the records through
                // one of them are a prefix of each list
                nbnd_p = 0;
                while (nbnd_p < nown && bnd[perm[p0 + nbnd_p]]) ++nbnd_p;
                ncell_a = 0;
                while (ncell_a < (int)lcell.size() && lo_c(lcell[ncell_a]) < nbnd_p) ++ncell_a;
                nhin_a = 0;
                while (nhin_a < (int)lhin.size() && lo_h(lhin[nhin_a]) < nbnd_p) ++nhin_a;
            }
            const int nlocal = nown + (int)halo.size();
            const int ncell = (int)lcell.size(), nhin = (int)lhin.size();
            const int nslot = 6 * ncell + 4 * nhin;
            if (nlocal > 65535 || nslot > 65535) {
                err = "patch too large for 16-bit local indices; lower patch_verts";
                return false;
            }
            // halo, gather pointers and gather entries of every patch start
            // on a 16-byte boundary, so a patch's lists can be bulk-copied
            while (L.halo.size() % 4) L.halo.push_back(0);
            while (L.csr_ptr.size() % 4) L.csr_ptr.push_back(0);
            while (L.csr_ent.size() % 8) L.csr_ent.push_back(0);
            PatchHdr ph{};
            ph.cloth = ci;
            ph.vbegin = vbase + p0;
            ph.nown = nown;
            ph.nlocal = nlocal;
            ph.halo_off = (int)L.halo.size();
            // records of every patch start on a group boundary (device format)
            while (L.cells.size() % kCellGroup) L.cells.push_back(pad_cell());
            ph.cell_off = (int)L.cells.size();
            ph.ncell = ncell;
            ph.hinge_off = (int)L.hinges.size();
            ph.nhinge = nhin;
            ph.csr_off = (int)L.csr_ptr.size();
            ph.ent_off = (int)L.csr_ent.size();
            ph.nslot = nslot;
            for (int n : halo) L.halo.push_back(vbase + n);
            for (int c : lcell) {
                const CellBuild& cb = cells[c];
                CellRec r = cb.rec;
                const uint32_t l0 = loc(cb.v[0]);
                auto lv = [&](int k) { return cb.v[k] >= 0 ? loc(cb.v[k]) : l0; };
                r.c01 = l0 | (lv(1) << 16);
                r.c23 = lv(2) | (lv(3) << 16);
                r.x12 = lv(4) | (lv(5) << 16);
                L.cells.push_back(r);
            }
            for (int q : lhin) {
                const int e = lone[q];
                HingeRec r{};
                r.w = make_float4(cd.w[4 * e], cd.w[4 * e + 1], cd.w[4 * e + 2], cd.w[4 * e + 3]);
                r.h2k = h2 * cd.bend_k[e];
                r.nrest = cd.n_rest[e];
                r.l01 = loc(cd.quads[4 * e]) | (loc(cd.quads[4 * e + 1]) << 16);
                r.l23 = loc(cd.quads[4 * e + 2]) | (loc(cd.quads[4 * e + 3]) << 16);
                L.hinges.push_back(r);
            }
            // gather lists: owned vertex l sums its outputs in global cell
            // order (outputs o0..o5 within a cell), then global lone-hinge
            // order -- independent of where the records sit in the patch, so
            // every patch size and launch structure adds in the same order
            std::vector<int> oc(ncell), oh(nhin);
            for (int q = 0; q < ncell; ++q) oc[q] = q;
            for (int q = 0; q < nhin; ++q) oh[q] = q;
            std::sort(oc.begin(), oc.end(), [&](int u, int w) { return lcell[u] < lcell[w]; });
            std::sort(oh.begin(), oh.end(), [&](int u, int w) { return lhin[u] < lhin[w]; });
            cnt.assign(nown + 1, 0);
            for (int lc = 0; lc < ncell; ++lc)
                for (int k = 0; k < 6; ++k) {
                    const int v = cells[lcell[lc]].v[k];
                    if (v >= 0 && (int)loc(v) < nown) cnt[loc(v) + 1]++;
                }
            for (int lh = 0; lh < nhin; ++lh)
                for (int a = 0; a < 4; ++a) {
                    const int l = (int)loc(cd.quads[4 * lone[lhin[lh]] + a]);
                    if (l < nown) cnt[l + 1]++;
                }
            for (int l = 0; l < nown; ++l) cnt[l + 1] += cnt[l];
            const size_t e0 = L.csr_ent.size();
            L.csr_ent.resize(e0 + cnt[nown]);
            for (int l = 0; l <= nown; ++l) L.csr_ptr.push_back(cnt[l]);
            std::vector<int> fill(cnt.begin(), cnt.end() - 1);
            // Vertex-major slot addressing (every kernel): contribution j of
            // owned vertex l at j*npad + l, so a warp's gather loads are
            // unit-stride and need no list entries; halo corners and absent
            // outputs get 0xffff and store nothing.  The per-vertex lists of
            // corner-major slot numbers (output k of cell lc at k*ncell + lc,
            // hinge corner a at 6*ncell + a*nhin + lh) stay on the host as the
            // record of each vertex's canonical summation order.
            int maxdeg = 0;
            for (int l = 0; l < nown; ++l) maxdeg = std::max(maxdeg, cnt[l + 1] - cnt[l]);
            const int npad = nown | 1;
            const long vm_nslot = (long)std::max(1, maxdeg) * npad;
            if (vm_nslot > 65535) {
                err = "patch too large for 16-bit slot addresses; lower patch_verts";
                return false;
            }
            std::vector<uint32_t> vm(nslot, 0xffffu);
            for (int lc : oc)
                for (int k = 0; k < 6; ++k) {
                    const int v = cells[lcell[lc]].v[k];
                    if (v < 0) continue;
                    const int l = (int)loc(v);
                    if (l < nown) {
                        vm[k * ncell + lc] = (uint32_t)((fill[l] - cnt[l]) * npad + l);
                        L.csr_ent[e0 + fill[l]++] = (uint16_t)(k * ncell + lc);
                    }
                }
            for (int lh : oh)
                for (int a = 0; a < 4; ++a) {
                    const int l = (int)loc(cd.quads[4 * lone[lhin[lh]] + a]);
                    if (l < nown) {
                        vm[6 * ncell + a * nhin + lh] = (uint32_t)((fill[l] - cnt[l]) * npad + l);
                        L.csr_ent[e0 + fill[l]++] = (uint16_t)(6 * ncell + a * nhin + lh);
                    }
                }
            for (int lc = 0; lc < ncell; ++lc) {
                CellRec& r = L.cells[ph.cell_off + lc];
                r.vm01 = vm[lc] | (vm[ncell + lc] << 16);
                r.vm23 = vm[2 * ncell + lc] | (vm[3 * ncell + lc] << 16);
                r.vm45 = vm[4 * ncell + lc] | (vm[5 * ncell + lc] << 16);
            }
            for (int lh = 0; lh < nhin; ++lh)
                L.hvm.push_back(make_uint2(vm[6 * ncell + lh] | (vm[6 * ncell + nhin + lh] << 16),
                                           vm[6 * ncell + 2 * nhin + lh] | (vm[6 * ncell + 3 * nhin + lh] << 16)));
            ph.vm_npad = npad;
            ph.vm_nslot = (int)vm_nslot;
            L.max_vm_slot = std::max(L.max_vm_slot, 32 * (size_t)nlocal + 12 * (size_t)vm_nslot);
            L.max_vm_nslot = std::max(L.max_vm_nslot, (int)vm_nslot);
            ph.nent = cnt[nown];
            ph.nbnd = nbnd_p;
            ph.ncell_a = ncell_a;
            ph.nhin_a = nhin_a;
            L.max_nent = std::max(L.max_nent, cnt[nown]);
            L.max_nhalo = std::max(L.max_nhalo, nlocal - nown);
            L.max_nlocal = std::max(L.max_nlocal, nlocal);
            L.max_nslot = std::max(L.max_nslot, nslot);
            L.max_nown = std::max(L.max_nown, nown);
            L.max_ncell = std::max(L.max_ncell, ncell);
            L.max_nhinge = std::max(L.max_nhinge, nhin);
            const size_t res = sizeof(CellRec) * (size_t)ncell + sizeof(HingeRec) * (size_t)nhin +
                               8 * (size_t)((nhin + 1) & ~1) + 32 * (size_t)nlocal + 12 * (size_t)vm_nslot +
                               4 * (size_t)(nown + 1);
            L.smem_resident = std::max(L.smem_resident, (res + 15) / 16 * 16);
            L.patches.push_back(ph);
        }
        info.patch_end = (int)L.patches.size();
        L.cinfo[ci] = info;
        vbase += N;
    }
    while (L.cells.size() % kCellGroup) L.cells.push_back(pad_cell());
    L.npatch = (int)L.patches.size();
    // a copy rounded up to 16 bytes never reads past the end
    for (int q = 0; q < 4; ++q) { L.halo.push_back(0); L.csr_ptr.push_back(0); }
    for (int q = 0; q < 8; ++q) L.csr_ent.push_back(0);
    // neighbour patches: the owners of each patch's halo vertices.  The
    // relation is symmetric (a record shared by two patches makes each read
    // the other's vertices), which the resident kernel's exchange relies on:
    // a patch overwrites its published d^(k-1) only after it has read d^k of
    // every patch that reads it (checked by check_layout).
    {
        std::vector<int> vpatch(ntot, -1);
        for (int p = 0; p < L.npatch; ++p)
            for (int l = 0; l < L.patches[p].nown; ++l) vpatch[L.patches[p].vbegin + l] = p;
        L.nbr_ptr.assign(1, 0);
        L.nbr.clear();
        std::vector<int> tmp;
        for (int p = 0; p < L.npatch; ++p) {
            const PatchHdr& h = L.patches[p];
            tmp.clear();
            for (int q = 0; q < h.nlocal - h.nown; ++q) tmp.push_back(vpatch[L.halo[h.halo_off + q]]);
            std::sort(tmp.begin(), tmp.end());
            tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
            L.nbr.insert(L.nbr.end(), tmp.begin(), tmp.end());
            L.nbr_ptr.push_back((int)L.nbr.size());
        }
    }
    // per-patch sweep kernels: y, d per local vertex and the vertex-major slots
    L.smem_bytes = (L.max_vm_slot + 15) / 16 * 16;
    return true;
}

// The properties of a layout that the sweep kernels rely on, checked on the
// host.  Returns an empty string, or the first violation found.
std::string check_layout(const std::vector<ClothSetup>& cl, const HostLayout& L)
{
    char msg[256];
    auto fail = [&](const char* fmt, auto... v) {
        std::snprintf(msg, sizeof msg, fmt, v...);
        return std::string(msg);
    };
    const int ntot = L.ntot;
    // 1. the reorder: a permutation within each cloth
    if ((int)L.perm_global.size() != ntot || (int)L.perm_local.size() != ntot || (int)L.vcloth.size() != ntot)
        return "reorder arrays do not hold every vertex";
    {
        std::vector<char> seen(ntot, 0);
        for (int ci = 0; ci < L.ncloth; ++ci) {
            const ClothInfo& info = L.cinfo[ci];
            if (info.nverts != cl[ci].mesh->N) return fail("cloth %d: %d vertices in the layout, %d in the mesh", ci,
                                                          info.nverts, cl[ci].mesh->N);
            for (int g = info.vbegin; g < info.vbegin + info.nverts; ++g) {
                const int o = L.perm_local[g];
                if (L.vcloth[g] != ci || o < 0 || o >= info.nverts || L.perm_global[g] != info.vbegin + o)
                    return fail("vertex %d: cloth or caller index out of place (cloth %d, index %d)", g, ci, o);
                if (seen[L.perm_global[g]]++) return fail("caller vertex %d appears twice (cloth %d)",
                                                          L.perm_global[g], ci);
            }
        }
    }
    // 2. the patches: consecutive runs of owned vertices, each inside its cloth
    std::vector<int> vpatch(ntot, -1);
    {
        int next = 0;
        for (int p = 0; p < L.npatch; ++p) {
            const PatchHdr& h = L.patches[p];
            const ClothInfo& info = L.cinfo[h.cloth];
            if (h.vbegin != next || h.nown < 1) return fail("patch %d: owns %d vertices from %d", p, h.nown, h.vbegin);
            if (p < info.patch_begin || p >= info.patch_end || h.vbegin < info.vbegin ||
                h.vbegin + h.nown > info.vbegin + info.nverts)
                return fail("patch %d: not inside cloth %d", p, h.cloth);
            for (int l = 0; l < h.nown; ++l) vpatch[h.vbegin + l] = p;
            next += h.nown;
        }
        if (next != ntot) return fail("patches own %d of %d vertices", next, ntot);
    }
    // vertices that some patch reads as a halo vertex (each entry range-checked
    // before it is used as an index)
    std::vector<char> in_halo(ntot, 0);
    for (int p = 0; p < L.npatch; ++p) {
        const PatchHdr& h = L.patches[p];
        if (h.halo_off < 0 || h.nlocal < h.nown || (size_t)h.halo_off + (size_t)(h.nlocal - h.nown) > L.halo.size())
            return fail("patch %d: halo list outside the halo array", p);
        for (int q = 0; q < h.nlocal - h.nown; ++q) {
            const int g = L.halo[h.halo_off + q];
            if (g < 0 || g >= ntot) return fail("patch %d: halo entry %d out of range (%d)", p, q, g);
            in_halo[g] = 1;
        }
    }

    std::vector<int> stamp(ntot, -1), nslot_of;
    std::vector<char> slot_seen;
    for (int p = 0; p < L.npatch; ++p) {
        const PatchHdr& h = L.patches[p];
        const ClothSetup& c = cl[h.cloth];
        const MeshData& m = *c.mesh;
        const Topology& tp = *c.topo;
        // 3. the halo: distinct vertices of the same cloth that the patch does
        //    not own, each owner on the patch's neighbour list
        for (int q = 0; q < h.nlocal - h.nown; ++q) {
            const int g = L.halo[h.halo_off + q];
            if (g < 0 || g >= ntot || L.vcloth[g] != h.cloth || vpatch[g] == p || stamp[g] == p)
                return fail("patch %d: halo entry %d (vertex %d) is foreign, owned or repeated", p, q, g);
            stamp[g] = p;
            const int* nb = L.nbr.data() + L.nbr_ptr[p];
            const int nnb = L.nbr_ptr[p + 1] - L.nbr_ptr[p];
            if (!std::binary_search(nb, nb + nnb, vpatch[g]))
                return fail("patch %d: owner %d of halo vertex %d is not a neighbour", p, vpatch[g], g);
        }
        //    and the neighbour relation is symmetric
        for (int j = L.nbr_ptr[p]; j < L.nbr_ptr[p + 1]; ++j) {
            const int q = L.nbr[j];
            if (q < 0 || q >= L.npatch || !std::binary_search(L.nbr.data() + L.nbr_ptr[q], L.nbr.data() + L.nbr_ptr[q + 1], p))
                return fail("patch %d: neighbour %d does not list it back", p, q);
        }
        // 4. boundary vertices first: every owned vertex another patch reads
        //    is published with the first nbnd
        for (int l = h.nbnd; l < h.nown; ++l)
            if (in_halo[h.vbegin + l]) return fail("patch %d: owned vertex %d is read by another patch but not among "
                                                   "the first %d", p, l, h.nbnd);
        // 5. the records: the patch's records start on a group boundary and
        //    lie inside the record array (the device format groups them by
        //    kCellGroup), local indices are in range, and every owned vertex's
        //    contributions j < deg are written to slot j*npad + l exactly
        //    once, by phase-A records (the prefix) if the vertex is a
        //    boundary one
        if (h.cell_off % kCellGroup != 0 || h.cell_off < 0 || h.ncell < 0 ||
            (size_t)h.cell_off + (size_t)(h.ncell + kCellGroup - 1) / kCellGroup * kCellGroup > L.cells.size())
            return fail("patch %d: records [%d, +%d) not group-aligned inside the record array", p, h.cell_off,
                        h.ncell);
        const int npad = h.vm_npad;
        if (npad < h.nown) return fail("patch %d: slot stride %d below %d owned vertices", p, npad, h.nown);
        const int* ptr = L.csr_ptr.data() + h.csr_off;
        int maxdeg = 0;
        for (int l = 0; l < h.nown; ++l) maxdeg = std::max(maxdeg, ptr[l + 1] - ptr[l]);
        if ((long)maxdeg * npad > h.vm_nslot) return fail("patch %d: %d slots, %d needed", p, h.vm_nslot, maxdeg * npad);
        slot_seen.assign(h.vm_nslot, 0);
        nslot_of.assign(h.nown, 0);
        auto slot = [&](uint32_t s, uint32_t l, bool phase_a) -> std::string {
            if (s == 0xffffu) return "";
            if ((int)l >= h.nown || (int)(s % npad) != (int)l || (int)(s / npad) >= ptr[l + 1] - ptr[l] ||
                (int)s >= h.vm_nslot)
                return fail("patch %d: slot %d does not belong to local vertex %d", p, (int)s, (int)l);
            if (slot_seen[s]++) return fail("patch %d: slot %d written twice (vertex %d)", p, (int)s, (int)l);
            if ((int)l < h.nbnd && !phase_a)
                return fail("patch %d: boundary vertex %d gets a contribution after phase A (slot %d)", p, (int)l,
                            (int)s);
            ++nslot_of[l];
            return "";
        };
        // triangles held by the patch's cells, as mesh triangle ids
        std::vector<int> held;
        auto caller = [&](uint32_t l) {
            const int g = (int)l < h.nown ? h.vbegin + (int)l : L.halo[h.halo_off + (int)l - h.nown];
            return L.perm_local[g];
        };
        auto find_tri = [&](int a, int b, int d) {
            for (int q = tp.vt_ptr[a]; q < tp.vt_ptr[a + 1]; ++q) {
                const int t = tp.vt[q];
                const int* v = &m.tris[3 * t];
                const bool hb = v[0] == b || v[1] == b || v[2] == b, hd = v[0] == d || v[1] == d || v[2] == d;
                if (hb && hd) return t;
            }
            return -1;
        };
        for (int q = 0; q < h.ncell; ++q) {
            const CellRec& r = L.cells[h.cell_off + q];
            const uint32_t cv[6] = {r.c01 & 0xffffu, r.c01 >> 16, r.c23 & 0xffffu, r.c23 >> 16, r.x12 & 0xffffu,
                                    r.x12 >> 16};
            const uint32_t sv[6] = {r.vm01 & 0xffffu, r.vm01 >> 16, r.vm23 & 0xffffu, r.vm23 >> 16, r.vm45 & 0xffffu,
                                    r.vm45 >> 16};
            for (int k = 0; k < 6; ++k) {
                if ((int)cv[k] >= h.nlocal) return fail("patch %d: cell %d names local vertex %d", p, q, (int)cv[k]);
                const std::string e = slot(sv[k], cv[k], q < h.ncell_a);
                if (!e.empty()) return e;
            }
            const int t0 = find_tri(caller(cv[0]), caller(cv[1]), caller(cv[2]));
            if (t0 < 0) return fail("patch %d: cell %d's first triangle is not a mesh triangle", p, q);
            held.push_back(t0);
            if (cv[3] != cv[0]) {   // paired: the second triangle shares the edge c0-c1
                const int t1 = find_tri(caller(cv[0]), caller(cv[1]), caller(cv[3]));
                if (t1 < 0) return fail("patch %d: cell %d's second triangle is not a mesh triangle", p, q);
                held.push_back(t1);
            }
        }
        for (int q = 0; q < h.nhinge; ++q) {
            const HingeRec& r = L.hinges[h.hinge_off + q];
            const uint2 vm = L.hvm[h.hinge_off + q];
            const uint32_t lv[4] = {r.l01 & 0xffffu, r.l01 >> 16, r.l23 & 0xffffu, r.l23 >> 16};
            const uint32_t sv[4] = {vm.x & 0xffffu, vm.x >> 16, vm.y & 0xffffu, vm.y >> 16};
            for (int a = 0; a < 4; ++a) {
                if ((int)lv[a] >= h.nlocal) return fail("patch %d: hinge %d names local vertex %d", p, q, (int)lv[a]);
                const std::string e = slot(sv[a], lv[a], q < h.nhin_a);
                if (!e.empty()) return e;
            }
        }
        for (int l = 0; l < h.nown; ++l)
            if (nslot_of[l] != ptr[l + 1] - ptr[l])
                return fail("patch %d: vertex %d has %d contributions written", p, l, nslot_of[l]);
        // 6. every triangle through an owned vertex is held once by the patch
        std::sort(held.begin(), held.end());
        if (std::adjacent_find(held.begin(), held.end()) != held.end())
            return fail("patch %d: a triangle is held twice", p);
        for (int l = 0; l < h.nown; ++l) {
            const int o = L.perm_local[h.vbegin + l];
            for (int q = tp.vt_ptr[o]; q < tp.vt_ptr[o + 1]; ++q)
                if (!std::binary_search(held.begin(), held.end(), tp.vt[q]))
                    return fail("patch %d: triangle %d through owned vertex %d is missing", p, tp.vt[q], l);
        }
    }
    return "";
}

}  // namespace pdg
