// Host-side constraint setup of the PD cloth solver: the Eigen-free
// restatement of the reference's CPU setup stage.
//   generate_grid           src/mesh_generator.cpp:6-91
//   precompute_rest_state   src/cloth_mesh.cpp:138-211
//   build_topology          src/mesh_topology.cpp:11-97
//   build_bend              src/sim_constraints.cpp:48-127
//   jacobi_diag             src/sim_constraints.cpp:133-192
//   load_obj                src/cloth_mesh.cpp:89-132
// All arithmetic is float, as in the reference.
#include "pdg_host.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <sstream>

namespace pdg {

namespace {

struct V3 {
    float x, y, z;
};
inline V3 at(const std::vector<float>& p, int i) { return {p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float len(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 scale(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 divide(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }

}  // namespace

void generate_grid(int nrows, int ncols, float size, int type,
                   std::vector<float>& pos, std::vector<int>& tris)
{
    const int cr = nrows - 1, cc = ncols - 1;
    pos.clear();
    tris.clear();
    pos.reserve(3 * (size_t)(nrows * ncols + (type == 3 ? cr * cc : 0)));
    for (int i = 0; i < nrows; ++i)
        for (int j = 0; j < ncols; ++j) {
            pos.push_back((float)j * size);
            pos.push_back(0.0f);
            pos.push_back((float)i * size);
        }
    if (type == 3)  // cell centres after the grid: index nrows*ncols + i*cc + j
        for (int i = 0; i < cr; ++i)
            for (int j = 0; j < cc; ++j) {
                pos.push_back(((float)j + 0.5f) * size);
                pos.push_back(0.0f);
                pos.push_back(((float)i + 0.5f) * size);
            }
    auto tri = [&](int a, int b, int c) { tris.push_back(a); tris.push_back(b); tris.push_back(c); };
    for (int i = 0; i < cr; ++i)
        for (int j = 0; j < cc; ++j) {
            const int tl = i * ncols + j, tr = tl + 1, bl = tl + ncols, br = bl + 1;
            if (type == 3) {
                const int c = nrows * ncols + i * cc + j;
                tri(tl, tr, c); tri(tr, br, c); tri(br, bl, c); tri(bl, tl, c);
                continue;
            }
            const bool backslash = type == 0 || (type == 1 && ((i + j) & 1) == 0);
            if (backslash) { tri(tl, tr, br); tri(tl, br, bl); }
            else           { tri(tl, tr, bl); tri(tr, br, bl); }
        }
}

void precompute_rest_state(MeshData& m)
{
    m.Dm_inv.assign(4 * (size_t)m.T, 0.0f);
    m.area.assign(m.T, 0.0f);
    m.mass.assign(m.N, 0.0f);
    for (int t = 0; t < m.T; ++t) {
        const int* v = &m.tris[3 * t];
        const V3 X0 = at(m.rest, v[0]);
        const V3 e1 = sub(at(m.rest, v[1]), X0), e2 = sub(at(m.rest, v[2]), X0);
        // In-plane orthonormal frame (b0, b1) of the rest triangle.
        const float l1 = len(e1);
        const V3 b0 = l1 > 0.0f ? divide(e1, l1) : V3{0.0f, 0.0f, 0.0f};
        const V3 o = sub(e2, scale(b0, dot(e2, b0)));
        const float lo = len(o);
        V3 b1;
        if (lo > 1e-10f) {
            b1 = divide(o, lo);
        } else {
            // degenerate rest triangle: any unit vector orthogonal to b0
            const bool x_smallest = std::fabs(b0.x) <= std::fabs(b0.y) && std::fabs(b0.x) <= std::fabs(b0.z);
            const V3 q = x_smallest ? V3{0.0f, -b0.z, b0.y} : V3{-b0.y, b0.x, 0.0f};
            const float lq = len(q);
            b1 = lq > 0.0f ? divide(q, lq) : V3{0.0f, 0.0f, 0.0f};
        }
        // Dm = [b0 b1]^T [e1 e2] and its cofactor inverse.
        const float a = dot(b0, e1), b = dot(b0, e2), c = dot(b1, e1), d = dot(b1, e2);
        const float det = a * d - c * b;
        const float inv = 1.0f / det;
        float* G = &m.Dm_inv[4 * t];
        G[0] = d * inv;   // g00
        G[1] = -c * inv;  // g10
        G[2] = -b * inv;  // g01
        G[3] = a * inv;   // g11
        const float A = 0.5f * std::fabs(det);
        m.area[t] = A;
        const float corner = m.density * A / 3.0f;
        m.mass[v[0]] += corner;
        m.mass[v[1]] += corner;
        m.mass[v[2]] += corner;
    }
}

void build_topology(const MeshData& m, Topology& t)
{
    // Sort the 3T directed triangle sides by their undirected key; within a
    // key the sort is stable in (triangle, side) order, so the first entry is
    // the first triangle that references the edge (tri_a) and the last the
    // last one (tri_b), matching the reference's map updates.
    const int S = 3 * m.T;
    std::vector<uint64_t> key(S);
    std::vector<int> order(S);
    for (int s = 0; s < S; ++s) {
        int a = m.tris[s], b = m.tris[(s / 3) * 3 + (s % 3 + 1) % 3];
        if (a > b) std::swap(a, b);
        key[s] = ((uint64_t)(uint32_t)a << 32) | (uint32_t)b;
        order[s] = s;
    }
    std::stable_sort(order.begin(), order.end(), [&](int p, int q) { return key[p] < key[q]; });
    t.edges.clear();
    t.rest_len.clear();
    t.num_inner = 0;
    for (int i = 0; i < S;) {
        int j = i;
        while (j + 1 < S && key[order[j + 1]] == key[order[i]]) ++j;
        const int v0 = (int)(key[order[i]] >> 32), v1 = (int)(key[order[i]] & 0xffffffffu);
        const int ta = order[i] / 3, tb = j > i ? order[j] / 3 : -1;
        t.edges.insert(t.edges.end(), {v0, v1, ta, tb});
        t.rest_len.push_back(len(sub(at(m.rest, v1), at(m.rest, v0))));
        if (tb != -1) ++t.num_inner;
        i = j + 1;
    }
    // vertex -> triangles, in triangle order
    t.vt_ptr.assign(m.N + 1, 0);
    for (int s = 0; s < S; ++s) t.vt_ptr[m.tris[s] + 1]++;
    for (int i = 0; i < m.N; ++i) t.vt_ptr[i + 1] += t.vt_ptr[i];
    t.vt.assign(S, 0);
    std::vector<int> fill(t.vt_ptr.begin(), t.vt_ptr.end() - 1);
    for (int s = 0; s < S; ++s) t.vt[fill[m.tris[s]]++] = s / 3;
    // triangle -> neighbour across the side opposite each corner
    t.tri_tri.assign(S, -1);
    const size_t nE = t.edges.size() / 4;
    for (size_t e = 0; e < nE; ++e) {
        const int v0 = t.edges[4 * e], v1 = t.edges[4 * e + 1], ta = t.edges[4 * e + 2], tb = t.edges[4 * e + 3];
        if (tb == -1) continue;
        for (int k = 0; k < 3; ++k) {
            const int va = m.tris[3 * ta + k];
            if (va != v0 && va != v1) { t.tri_tri[3 * ta + k] = tb; break; }
        }
        for (int k = 0; k < 3; ++k) {
            const int vb = m.tris[3 * tb + k];
            if (vb != v0 && vb != v1) { t.tri_tri[3 * tb + k] = ta; break; }
        }
    }
}

namespace {
int opposite(const MeshData& m, int tri, int v0, int v1)
{
    for (int k = 0; k < 3; ++k) {
        const int v = m.tris[3 * tri + k];
        if (v != v0 && v != v1) return v;
    }
    return -1;
}
float heron(float a, float b, float c)
{
    const float s = 0.5f * (a + b + c);
    const float q = s * (s - a) * (s - b) * (s - c);
    return q > 0.0f ? std::sqrt(q) : 0.0f;
}
}  // namespace

void build_bend(const MeshData& m, const Topology& t, float k, ConstraintData& c)
{
    c.quads.clear(); c.w.clear(); c.n_rest.clear(); c.bend_k.clear();
    const size_t nE = t.edges.size() / 4;
    for (size_t e = 0; e < nE; ++e) {
        const int v0 = t.edges[4 * e], v1 = t.edges[4 * e + 1];
        const int ta = t.edges[4 * e + 2], tb = t.edges[4 * e + 3];
        if (tb == -1) continue;  // boundary edge: no hinge
        const int v2 = opposite(m, ta, v0, v1), v3 = opposite(m, tb, v0, v1);
        if (v2 < 0 || v3 < 0) continue;
        const V3 X0 = at(m.rest, v0), X1 = at(m.rest, v1), X2 = at(m.rest, v2), X3 = at(m.rest, v3);
        const float l01 = len(sub(X1, X0)), l02 = len(sub(X2, X0)), l03 = len(sub(X3, X0));
        const float l12 = len(sub(X2, X1)), l13 = len(sub(X3, X1));
        const float A0 = heron(l01, l02, l12), A1 = heron(l01, l03, l13);
        if (A0 < 1e-10f || A1 < 1e-10f) continue;  // degenerate wing
        // cotangents of the angles facing the shared edge's endpoints
        const float c02 = (l01 * l01 + l12 * l12 - l02 * l02) / (4.0f * A0);  // at v1, wing a
        const float c12 = (l01 * l01 + l02 * l02 - l12 * l12) / (4.0f * A0);  // at v0, wing a
        const float c03 = (l01 * l01 + l13 * l13 - l03 * l03) / (4.0f * A1);  // at v1, wing b
        const float c13 = (l01 * l01 + l03 * l03 - l13 * l13) / (4.0f * A1);  // at v0, wing b
        const float w[4] = {c02 + c03, c12 + c13, -(c02 + c12), -(c03 + c13)};
        const V3 er = {w[0] * X0.x + w[1] * X1.x + w[2] * X2.x + w[3] * X3.x,
                       w[0] * X0.y + w[1] * X1.y + w[2] * X2.y + w[3] * X3.y,
                       w[0] * X0.z + w[1] * X1.z + w[2] * X2.z + w[3] * X3.z};
        c.quads.insert(c.quads.end(), {v0, v1, v2, v3});
        c.w.insert(c.w.end(), w, w + 4);
        c.n_rest.push_back(len(er));
        c.bend_k.push_back(k);
    }
}

void jacobi_diag(const MeshData& m, const ConstraintData& c, float dt, std::vector<float>& diag)
{
    const float h2 = dt * dt;
    diag.assign(m.mass.begin(), m.mass.end());
    const int T = std::min<int>(m.T, (int)c.k_stretch.size());
    for (int t = 0; t < T; ++t) {
        const float wA = c.k_stretch[t] * m.area[t];
        const float* G = &m.Dm_inv[4 * t];
        const float s0 = G[0] + G[1], s1 = G[2] + G[3];
        diag[m.tris[3 * t + 0]] += h2 * wA * (s0 * s0 + s1 * s1);
        diag[m.tris[3 * t + 1]] += h2 * wA * (G[0] * G[0] + G[2] * G[2]);
        diag[m.tris[3 * t + 2]] += h2 * wA * (G[1] * G[1] + G[3] * G[3]);
    }
    const size_t E = c.bend_k.size();
    for (size_t e = 0; e < E; ++e)
        for (int i = 0; i < 4; ++i) {
            const float wi = c.w[4 * e + i];
            diag[c.quads[4 * e + i]] += h2 * c.bend_k[e] * wi * wi;
        }
}

bool load_obj(const std::string& path, std::vector<float>& pos, std::vector<int>& tris, std::string& err)
{
    std::ifstream in(path);
    if (!in) { err = "cannot open '" + path + "'"; return false; }
    pos.clear();
    tris.clear();
    std::string line;
    std::vector<int> face;
    while (std::getline(in, line)) {
        if (line.empty() || line[0] == '#') continue;
        std::istringstream ls(line);
        std::string tag;
        ls >> tag;
        if (tag == "v") {
            float x = 0, y = 0, z = 0;
            ls >> x >> y >> z;
            pos.insert(pos.end(), {x, y, z});
        } else if (tag == "f") {
            face.clear();
            std::string tok;
            while (ls >> tok) face.push_back(std::atoi(tok.c_str()) - 1);  // "i/t/n" -> i, 1-based
            for (size_t k = 1; k + 1 < face.size(); ++k)                    // fan
                tris.insert(tris.end(), {face[0], face[k], face[k + 1]});
        }
    }
    if (pos.empty() || tris.empty()) { err = "empty mesh in '" + path + "'"; return false; }
    const int N = (int)(pos.size() / 3);
    for (int v : tris)
        if (v < 0 || v >= N) { err = "face index out of range in '" + path + "'"; return false; }
    return true;
}

uint64_t splitmix64(uint64_t& s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

double gaussian(uint64_t& s)
{
    // Box-Muller on two 53-bit uniforms in (0, 1]
    const double u1 = ((splitmix64(s) >> 11) + 1) * (1.0 / 9007199254740992.0);
    const double u2 = ((splitmix64(s) >> 11) + 1) * (1.0 / 9007199254740992.0);
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

}  // namespace pdg
