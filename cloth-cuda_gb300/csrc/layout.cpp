// Host-side construction of the device layout: Morton reorder of every
// cloth, cut into patches, local triangle/hinge records with 16-bit vertex
// references, and per-vertex gather lists (CSR) over contribution slots.
#include "pdg_solver.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace pdg {

namespace {

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
        const int N = m.N, T = m.T, E = (int)cd.bend_k.size();
        std::vector<int> perm, iperm(N);
        morton_order(m, perm);
        for (int i = 0; i < N; ++i) iperm[perm[i]] = i;
        // A vertex is "boundary" when a triangle or hinge through it has a
        // corner in another patch (it is then in that patch's halo).  Within
        // each patch the boundary vertices go first, so a kernel can finish
        // and publish them before the interior.
        std::vector<char> bnd(N, 0);
        {
            auto mark = [&](const int* v, int n) {
                const int p = iperm[v[0]] / patch_verts;
                bool span = false;
                for (int a = 1; a < n; ++a) span = span || iperm[v[a]] / patch_verts != p;
                if (span)
                    for (int a = 0; a < n; ++a) bnd[v[a]] = 1;
            };
            for (int t = 0; t < T; ++t) mark(&m.tris[3 * t], 3);
            for (int e = 0; e < E; ++e) mark(&cd.quads[4 * e], 4);
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

        // vertex -> hinge lists
        std::vector<int> vh_ptr(N + 1, 0), vh(4 * (size_t)E);
        for (int e = 0; e < E; ++e)
            for (int a = 0; a < 4; ++a) vh_ptr[cd.quads[4 * e + a] + 1]++;
        for (int i = 0; i < N; ++i) vh_ptr[i + 1] += vh_ptr[i];
        {
            std::vector<int> f(vh_ptr.begin(), vh_ptr.end() - 1);
            for (int e = 0; e < E; ++e)
                for (int a = 0; a < 4; ++a) vh[f[cd.quads[4 * e + a]]++] = e;
        }

        std::vector<int> tmark(T, -1), hmark(E, -1), vmark(N, -1), vloc(N, 0);
        std::vector<int> ltri, lhin, halo, cnt;
        const float h2 = cfg.dt * cfg.dt;
        for (int p0 = 0; p0 < N; p0 += patch_verts) {
            const int p1 = std::min(N, p0 + patch_verts);
            const int nown = p1 - p0;
            const int stamp = (int)L.patches.size();
            ltri.clear(); lhin.clear(); halo.clear();
            int nbnd_p = 0, ntri_a = 0, nhin_a = 0;
            for (int l = 0; l < nown; ++l) {
                const int o = perm[p0 + l];
                for (int q = tp.vt_ptr[o]; q < tp.vt_ptr[o + 1]; ++q) {
                    const int t = tp.vt[q];
                    if (tmark[t] != stamp) { tmark[t] = stamp; ltri.push_back(t); }
                }
                for (int q = vh_ptr[o]; q < vh_ptr[o + 1]; ++q) {
                    const int e = vh[q];
                    if (hmark[e] != stamp) { hmark[e] = stamp; lhin.push_back(e); }
                }
            }
            std::sort(ltri.begin(), ltri.end());
            std::sort(lhin.begin(), lhin.end());
            auto touch = [&](int o) {
                const int n = iperm[o];
                if (n >= p0 && n < p1) return;
                if (vmark[n] != stamp) { vmark[n] = stamp; halo.push_back(n); }
            };
            for (int t : ltri)
                for (int a = 0; a < 3; ++a) touch(m.tris[3 * t + a]);
            for (int e : lhin)
                for (int a = 0; a < 4; ++a) touch(cd.quads[4 * e + a]);
            std::sort(halo.begin(), halo.end());
            for (int l = 0; l < nown; ++l) vloc[p0 + l] = l;
            for (size_t q = 0; q < halo.size(); ++q) vloc[halo[q]] = nown + (int)q;
            // record placement follows the Morton order of the lowest local
            // corner, so the lanes of a warp touch neighbouring vertices and
            // neighbouring slots (fewer shared-memory bank conflicts); the
            // summation order is fixed separately below
            {
                auto lo_t = [&](int t) {
                    return std::min(vloc[iperm[m.tris[3 * t]]],
                                    std::min(vloc[iperm[m.tris[3 * t + 1]]], vloc[iperm[m.tris[3 * t + 2]]]));
                };
                auto lo_h = [&](int e) {
                    int lo = vloc[iperm[cd.quads[4 * e]]];
                    for (int a = 1; a < 4; ++a) lo = std::min(lo, vloc[iperm[cd.quads[4 * e + a]]]);
                    return lo;
                };
                std::stable_sort(ltri.begin(), ltri.end(), [&](int u, int w) { return lo_t(u) < lo_t(w); });
                std::stable_sort(lhin.begin(), lhin.end(), [&](int u, int w) { return lo_h(u) < lo_h(w); });
                // boundary vertices are local 0..nbnd-1; the records through
                // one of them are a prefix of each list
                nbnd_p = 0;
                while (nbnd_p < nown && bnd[perm[p0 + nbnd_p]]) ++nbnd_p;
                ntri_a = 0;
                while (ntri_a < (int)ltri.size() && lo_t(ltri[ntri_a]) < nbnd_p) ++ntri_a;
                nhin_a = 0;
                while (nhin_a < (int)lhin.size() && lo_h(lhin[nhin_a]) < nbnd_p) ++nhin_a;
            }
            const int nlocal = nown + (int)halo.size();
            const int ntri = (int)ltri.size(), nhin = (int)lhin.size();
            const int nslot = 3 * ntri + 4 * nhin;
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
            ph.tri_off = (int)L.tris.size();
            ph.ntri = ntri;
            ph.hinge_off = (int)L.hinges.size();
            ph.nhinge = nhin;
            ph.csr_off = (int)L.csr_ptr.size();
            ph.ent_off = (int)L.csr_ent.size();
            ph.nslot = nslot;
            for (int n : halo) L.halo.push_back(vbase + n);
            auto loc = [&](int o) { return (uint32_t)vloc[iperm[o]]; };
            for (int t : ltri) {
                TriRec r{};
                const float* G = &m.Dm_inv[4 * t];
                r.G = make_float4(G[0], G[1], G[2], G[3]);
                const float k = t < (int)cd.k_stretch.size() ? cd.k_stretch[t] : 0.f;
                r.h2wA = h2 * (k * m.area[t]);
                r.l01 = loc(m.tris[3 * t]) | (loc(m.tris[3 * t + 1]) << 16);
                r.l2 = loc(m.tris[3 * t + 2]);
                L.tris.push_back(r);
            }
            for (int e : lhin) {
                HingeRec r{};
                r.w = make_float4(cd.w[4 * e], cd.w[4 * e + 1], cd.w[4 * e + 2], cd.w[4 * e + 3]);
                r.h2k = h2 * cd.bend_k[e];
                r.nrest = cd.n_rest[e];
                r.l01 = loc(cd.quads[4 * e]) | (loc(cd.quads[4 * e + 1]) << 16);
                r.l23 = loc(cd.quads[4 * e + 2]) | (loc(cd.quads[4 * e + 3]) << 16);
                L.hinges.push_back(r);
            }
            // gather lists: owned vertex l sums the slots of its corners in
            // global triangle order, then global hinge order -- independent
            // of where the records sit in the patch, so every patch size and
            // launch structure adds in the same order
            std::vector<int> ot(ntri), oh(nhin);
            for (int q = 0; q < ntri; ++q) ot[q] = q;
            for (int q = 0; q < nhin; ++q) oh[q] = q;
            std::sort(ot.begin(), ot.end(), [&](int u, int w) { return ltri[u] < ltri[w]; });
            std::sort(oh.begin(), oh.end(), [&](int u, int w) { return lhin[u] < lhin[w]; });
            cnt.assign(nown + 1, 0);
            for (int lt = 0; lt < ntri; ++lt)
                for (int a = 0; a < 3; ++a) {
                    const int l = (int)loc(m.tris[3 * ltri[lt] + a]);
                    if (l < nown) cnt[l + 1]++;
                }
            for (int lh = 0; lh < nhin; ++lh)
                for (int a = 0; a < 4; ++a) {
                    const int l = (int)loc(cd.quads[4 * lhin[lh] + a]);
                    if (l < nown) cnt[l + 1]++;
                }
            for (int l = 0; l < nown; ++l) cnt[l + 1] += cnt[l];
            const size_t e0 = L.csr_ent.size();
            L.csr_ent.resize(e0 + cnt[nown]);
            for (int l = 0; l <= nown; ++l) L.csr_ptr.push_back(cnt[l]);
            std::vector<int> fill(cnt.begin(), cnt.end() - 1);
            // Two slot addressings hold the same contributions.  Corner-major
            // (resident and streaming kernels, summed through the gather
            // lists): triangle corner a at a*ntri + lt, hinge corner a at
            // 3*ntri + a*nhin + lh.  Vertex-major (per-patch sweep kernels):
            // contribution j of owned vertex l at j*npad + l, so a warp's
            // gather loads are unit-stride and need no list entries; halo
            // corners get 0xffff and store nothing.
            int maxdeg = 0;
            for (int l = 0; l < nown; ++l) maxdeg = std::max(maxdeg, cnt[l + 1] - cnt[l]);
            const int npad = nown | 1;
            const long vm_nslot = (long)std::max(1, maxdeg) * npad;
            if (vm_nslot > 65535) {
                err = "patch too large for 16-bit slot addresses; lower patch_verts";
                return false;
            }
            std::vector<uint32_t> vm(nslot, 0xffffu);
            for (int lt : ot)
                for (int a = 0; a < 3; ++a) {
                    const int l = (int)loc(m.tris[3 * ltri[lt] + a]);
                    if (l < nown) {
                        vm[a * ntri + lt] = (uint32_t)((fill[l] - cnt[l]) * npad + l);
                        L.csr_ent[e0 + fill[l]++] = (uint16_t)(a * ntri + lt);
                    }
                }
            for (int lh : oh)
                for (int a = 0; a < 4; ++a) {
                    const int l = (int)loc(cd.quads[4 * lhin[lh] + a]);
                    if (l < nown) {
                        vm[3 * ntri + a * nhin + lh] = (uint32_t)((fill[l] - cnt[l]) * npad + l);
                        L.csr_ent[e0 + fill[l]++] = (uint16_t)(3 * ntri + a * nhin + lh);
                    }
                }
            for (int lt = 0; lt < ntri; ++lt) {
                TriRec& r = L.tris[ph.tri_off + lt];
                r.l2 |= vm[lt] << 16;
                r.vm12 = vm[ntri + lt] | (vm[2 * ntri + lt] << 16);
            }
            for (int lh = 0; lh < nhin; ++lh)
                L.hvm.push_back(make_uint2(vm[3 * ntri + lh] | (vm[3 * ntri + nhin + lh] << 16),
                                           vm[3 * ntri + 2 * nhin + lh] | (vm[3 * ntri + 3 * nhin + lh] << 16)));
            ph.vm_npad = npad;
            ph.vm_nslot = (int)vm_nslot;
            L.max_vm_slot = std::max(L.max_vm_slot, 32 * (size_t)nlocal + 12 * (size_t)vm_nslot);
            ph.nent = cnt[nown];
            ph.nbnd = nbnd_p;
            ph.ntri_a = ntri_a;
            ph.nhin_a = nhin_a;
            L.max_nent = std::max(L.max_nent, cnt[nown]);
            L.max_nhalo = std::max(L.max_nhalo, nlocal - nown);
            L.max_nlocal = std::max(L.max_nlocal, nlocal);
            L.max_nslot = std::max(L.max_nslot, nslot);
            L.max_nown = std::max(L.max_nown, nown);
            L.max_ntri = std::max(L.max_ntri, ntri);
            L.max_nhinge = std::max(L.max_nhinge, nhin);
            const size_t res = 32 * (size_t)nlocal + 12 * (size_t)nslot + 4 * (size_t)(nown + 1) + 2 * (size_t)cnt[nown];
            L.smem_resident = std::max(L.smem_resident, (res + 15) / 16 * 16);
            L.patches.push_back(ph);
        }
        info.patch_end = (int)L.patches.size();
        L.cinfo[ci] = info;
        vbase += N;
    }
    L.npatch = (int)L.patches.size();
    // a copy rounded up to 16 bytes never reads past the end
    for (int q = 0; q < 4; ++q) { L.halo.push_back(0); L.csr_ptr.push_back(0); }
    for (int q = 0; q < 8; ++q) L.csr_ent.push_back(0);
    // neighbour patches: the owners of each patch's halo vertices
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

}  // namespace pdg
