// Learned warm start: host side and C ABI (no counterpart in the reference).
// The kernels live in gnn_kernels.cuh; this file owns the parameters, the
// activation buffers, the training step and the binding to a solver.
#include "gnn_kernels.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

using namespace pdg;
using namespace pdg::gnn;

#define GK(call)                                                                                \
    do {                                                                                        \
        const cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                                  \
            return set_error(e_ == cudaErrorMemoryAllocation ? PDG_ERR_ALLOC : PDG_ERR_CUDA,    \
                             "warm start: %s: %s", #call, cudaGetErrorString(e_));              \
    } while (0)

struct pdg_warmstart {
    Layout lay;
    long long t = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    DevBuf<float> p, g, m, v, bdp;
    DevBuf<float> part;   // per-block partial weight gradients (summed in a fixed order)
    DevBuf<bf16> wbuf;
    Bf16Weights W{};
    // graph and activations
    int N = 0, E = 0;
    DevBuf<int> ptr, adj, rev;
    DevBuf<float> rest, deg_inv;
    DevBuf<float4> ef, stat, Xn, Vn, Dn;
    DevBuf<float> ew;     // per directed edge: weight of the energy-norm term of the loss
    DevBuf<bf16> xin, cat[L], pq[L], uo[L], hfin;
    DevBuf<float> out, target, freew, dout, dh, dtmp, dcat, dpq;
    DevBuf<double> loss;
    float smooth = 0.f;   // weight of the neighbour-difference term of the loss
    int energy = 0;       // 1: that term weighted by the PD system's stiffness per edge
    // sweeps each start runs before the judge compares them; 1: the starts'
    // own residuals, which each chain's first sweep evaluates
    int judge = 1;
    pdg_solver* solver = nullptr;
    ~pdg_warmstart()
    {
        if (own_stream && stream) cudaStreamDestroy(stream);
    }
};

namespace {

inline int nb(long long n, int b) { return (int)((n + b - 1) / b); }

constexpr int kWgradBlocks = 304;        // at most, blocks of a weight-gradient reduction
constexpr int kMsgBwdBlocks = 4 * 152;   // at most, blocks of the message backward

int refresh_bf16(pdg_warmstart* w, cudaStream_t st)
{
    const Layout& y = w->lay;
    const float* p = w->p.p;
    k_to_bf16<<<nb(H * NF, 256), 256, 0, st>>>(p + y.We, H, NF, w->W.We, NFP, nullptr, 0);
    for (int l = 0; l < L; ++l) {
        k_to_bf16<<<nb(H * H, 256), 256, 0, st>>>(p + y.A[l], H, H, w->W.AB[l], H, w->W.ABt[l], 2 * H);
        k_to_bf16<<<nb(H * H, 256), 256, 0, st>>>(p + y.B[l], H, H, w->W.AB[l] + H * H, H, w->W.ABt[l] + H, 2 * H);
        k_to_bf16<<<nb(H * 2 * H, 256), 256, 0, st>>>(p + y.U[l], H, 2 * H, w->W.U[l], 2 * H, w->W.Ut[l], H);
    }
    k_to_bf16<<<nb(NO * H, 256), 256, 0, st>>>(p + y.Wd, NO, H, w->W.Wd, H, w->W.Wdt, 16);
    GK(cudaMemcpyAsync(w->bdp.p, p + y.bd, sizeof(float) * NO, cudaMemcpyDeviceToDevice, st));
    GK(cudaGetLastError());
    return PDG_OK;
}

int alloc_params(pdg_warmstart* w)
{
    const int n = w->lay.total;
    GK(w->p.alloc(n)); GK(w->g.alloc(n)); GK(w->m.alloc(n)); GK(w->v.alloc(n)); GK(w->bdp.alloc(16));
    GK(w->part.alloc(std::max((size_t)kWgradBlocks * (2 * H * H + 2 * H), (size_t)kMsgBwdBlocks * H * (EF + 1))));
    // bf16 copies: We 64x16, per layer AB 128x64, ABt 64x128, U 64x128, Ut 128x64, Wd 16x64, Wdt 64x16
    const size_t sizes[] = {(size_t)H * NFP, 2u * H * H, 2u * H * H, 2u * H * H, 2u * H * H, 16u * H, (size_t)H * 16};
    size_t total = sizes[0] + L * (sizes[1] + sizes[2] + sizes[3] + sizes[4]) + sizes[5] + sizes[6];
    GK(w->wbuf.alloc(total));
    GK(cudaMemsetAsync(w->wbuf.p, 0, sizeof(bf16) * total, w->stream));
    GK(cudaMemsetAsync(w->bdp.p, 0, sizeof(float) * 16, w->stream));
    bf16* q = w->wbuf.p;
    w->W.We = q; q += sizes[0];
    for (int l = 0; l < L; ++l) {
        w->W.AB[l] = q; q += sizes[1];
        w->W.ABt[l] = q; q += sizes[2];
        w->W.U[l] = q; q += sizes[3];
        w->W.Ut[l] = q; q += sizes[4];
    }
    w->W.Wd = q; q += sizes[5];
    w->W.Wdt = q;
    GK(cudaMemsetAsync(w->g.p, 0, sizeof(float) * n, w->stream));
    GK(cudaMemsetAsync(w->m.p, 0, sizeof(float) * n, w->stream));
    GK(cudaMemsetAsync(w->v.p, 0, sizeof(float) * n, w->stream));
    return PDG_OK;
}

// activation buffers for N nodes and E directed edges
int alloc_graph(pdg_warmstart* w, int N, int E)
{
    w->N = N; w->E = E;
    GK(w->ptr.alloc(N + 1)); GK(w->adj.alloc(E)); GK(w->rev.alloc(E));
    GK(w->rest.alloc(E)); GK(w->deg_inv.alloc(N)); GK(w->ef.alloc(E)); GK(w->stat.alloc(N));
    GK(w->Xn.alloc(N)); GK(w->Vn.alloc(N)); GK(w->Dn.alloc(N)); GK(w->ew.alloc(E));
    GK(w->xin.alloc((size_t)N * NFP));
    for (int l = 0; l < L; ++l) {
        GK(w->cat[l].alloc((size_t)N * 2 * H)); GK(w->pq[l].alloc((size_t)N * 2 * H)); GK(w->uo[l].alloc((size_t)N * H));
    }
    GK(w->hfin.alloc((size_t)N * H));
    GK(w->out.alloc((size_t)N * 16)); GK(w->target.alloc((size_t)N * 3)); GK(w->freew.alloc(N));
    GK(w->dout.alloc((size_t)N * 16)); GK(w->dh.alloc((size_t)N * H)); GK(w->dtmp.alloc((size_t)N * H));
    GK(w->dcat.alloc((size_t)N * 2 * H)); GK(w->dpq.alloc((size_t)N * 2 * H)); GK(w->loss.alloc(1));
    return PDG_OK;
}

// The network on the current features for training: every activation the
// backward pass needs is kept (h and a per layer, P and Q, the update's ReLU
// output, the last h and the decoder output).  Inference runs the fused
// kernels instead (warm_infer_enqueue), with bitwise the same start offsets.
int forward(pdg_warmstart* w, cudaStream_t st)
{
    const int N = w->N;
    const Layout& y = w->lay;
    const float* p = w->p.p;
    gemm<bf16, NFP, H, EPI_RELU | EPI_STORE1>(st, w->xin.p, NFP, N, w->W.We, p + y.be, nullptr, 0, w->cat[0].p, 2 * H,
                                              nullptr, 0, nullptr, 0);
    for (int l = 0; l < L; ++l) {
        gemm<bf16, H, 2 * H, EPI_STORE1>(st, w->cat[l].p, 2 * H, N, w->W.AB[l], nullptr, nullptr, 0, w->pq[l].p, 2 * H,
                                         nullptr, 0, nullptr, 0);
        k_msg_fwd<<<msg_grid(N), 256, 0, st>>>(N, w->ptr.p, w->adj.p, w->ef.p, w->deg_inv.p, w->pq[l].p,
                                                             p + y.C[l], p + y.c[l], w->cat[l].p);
        bf16* next = l + 1 < L ? w->cat[l + 1].p : w->hfin.p;
        const int ldn = l + 1 < L ? 2 * H : H;
        // h <- h + relu(U [h; a] + u): the residual h is the A operand's
        // first H columns
        gemm<bf16, 2 * H, H, EPI_RELU | EPI_STORE1 | EPI_RESIDA>(st, w->cat[l].p, 2 * H, N, w->W.U[l], p + y.u[l],
                                                                 nullptr, 0, w->uo[l].p, H, next, ldn, nullptr, 0);
    }
    gemm<bf16, H, 16, EPI_STOREF>(st, w->hfin.p, H, N, w->W.Wd, w->bdp.p, nullptr, 0, nullptr, 0, nullptr, 0,
                                  w->out.p, 16);
    GK(cudaGetLastError());
    return PDG_OK;
}

int wgrad_grid(int M) { return std::max(1, std::min(kWgradBlocks, nb(M, 32))); }

// dW (nout x K) and db (nout, may be null) of dY^T X over M rows: block
// partial sums, then their sum in a fixed order
template <typename TY, typename TX>
void wgrad(pdg_warmstart* w, const TY* dY, int ldy, int nout, const TX* X, int ldx, int K, int M, float* dW,
           float* db, cudaStream_t st)
{
    const int gw = wgrad_grid(M);
    k_wgrad<TY, TX><<<gw, 256, 0, st>>>(dY, ldy, nout, X, ldx, K, M, w->part.p);
    k_sum_parts<<<nb(nout * K + nout, 256), 256, 0, st>>>(w->part.p, gw, nout * K, nout, dW, db);
}

// gradients of the loss w.r.t. all parameters into w->g (zeroed here);
// loss accumulated into w->loss; ew: per-edge weights of the smoothness term
// (null: 1)
int backward(pdg_warmstart* w, float inv_cnt, const float* ew, cudaStream_t st)
{
    const int N = w->N;
    const Layout& y = w->lay;
    const float* p = w->p.p;
    float* g = w->g.p;
    GK(cudaMemsetAsync(g, 0, sizeof(float) * y.total, st));
    GK(cudaMemsetAsync(w->loss.p, 0, sizeof(double), st));
    k_loss<<<nb(N, 256), 256, 0, st>>>(N, w->out.p, w->target.p, w->freew.p, w->ptr.p, w->adj.p, ew, w->smooth,
                                       inv_cnt, w->dout.p, w->loss.p);
    wgrad<float, bf16>(w, w->dout.p, 16, NO, w->hfin.p, H, H, N, g + y.Wd, g + y.bd, st);
    gemm<float, 16, H, EPI_STOREF>(st, w->dout.p, 16, N, w->W.Wdt, nullptr, nullptr, 0, nullptr, 0, nullptr, 0, w->dh.p,
                                   H);
    for (int l = L - 1; l >= 0; --l) {
        k_relu_bwd<<<nb((long long)N * H, 256), 256, 0, st>>>(N, H, w->dh.p, H, w->uo[l].p, H, w->dtmp.p, H);
        wgrad<float, bf16>(w, w->dtmp.p, H, H, w->cat[l].p, 2 * H, 2 * H, N, g + y.U[l], g + y.u[l], st);
        gemm<float, H, 2 * H, EPI_STOREF>(st, w->dtmp.p, H, N, w->W.Ut[l], nullptr, nullptr, 0, nullptr, 0, nullptr, 0,
                                          w->dcat.p, 2 * H);
        k_add<<<nb((long long)N * H, 256), 256, 0, st>>>(N, H, w->dcat.p, 2 * H, w->dh.p, H);
        const int gm = std::max(1, std::min(kMsgBwdBlocks, nb(N, 8)));
        k_msg_bwd<<<gm, 256, 0, st>>>(N, w->ptr.p, w->adj.p, w->rev.p, w->ef.p, w->deg_inv.p, w->pq[l].p, p + y.C[l],
                                      p + y.c[l], w->dcat.p, w->dpq.p, w->part.p);
        k_sum_parts<<<nb(H * (EF + 1), 256), 256, 0, st>>>(w->part.p, gm, H * EF, H, g + y.C[l], g + y.c[l]);
        wgrad<float, bf16>(w, w->dpq.p, 2 * H, 2 * H, w->cat[l].p, 2 * H, H, N, g + y.A[l], nullptr, st);
        gemm<float, 2 * H, H, EPI_ACCF>(st, w->dpq.p, 2 * H, N, w->W.ABt[l], nullptr, nullptr, 0, nullptr, 0, nullptr, 0,
                                        w->dh.p, H);
    }
    k_relu_bwd<<<nb((long long)N * H, 256), 256, 0, st>>>(N, H, w->dh.p, H, w->cat[0].p, 2 * H, w->dtmp.p, H);
    wgrad<float, bf16>(w, w->dtmp.p, H, H, w->xin.p, NFP, NF, N, g + y.We, g + y.be, st);
    GK(cudaGetLastError());
    return PDG_OK;
}

int adam_step(pdg_warmstart* w, float lr, cudaStream_t st)
{
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    w->t += 1;
    const float bc1 = 1.f - (float)std::pow((double)b1, (double)w->t);
    const float bc2 = 1.f - (float)std::pow((double)b2, (double)w->t);
    k_adam<<<nb(w->lay.total, 256), 256, 0, st>>>(w->lay.total, w->p.p, w->g.p, w->m.p, w->v.p, lr, b1, b2, eps, bc1,
                                                  bc2);
    GK(cudaGetLastError());
    return refresh_bf16(w, st);
}

// reverse-edge index of a symmetric CSR; false if some edge has no reverse
bool reverse_edges(int N, const std::vector<int>& ptr, const std::vector<int>& adj, std::vector<int>& rev)
{
    rev.assign(adj.size(), -1);
    for (int i = 0; i < N; ++i)
        for (int e = ptr[i]; e < ptr[i + 1]; ++e) {
            const int j = adj[e];
            if (j < 0 || j >= N) return false;
            for (int f = ptr[j]; f < ptr[j + 1]; ++f)
                if (adj[f] == i) { rev[e] = f; break; }
            if (rev[e] < 0) return false;
        }
    return true;
}

int upload_graph(pdg_warmstart* w, const std::vector<int>& ptr, const std::vector<int>& adj, cudaStream_t st)
{
    const int N = (int)ptr.size() - 1;
    std::vector<int> rev;
    if (!reverse_edges(N, ptr, adj, rev)) return set_error(PDG_ERR_ARG, "warm start: adjacency is not symmetric");
    std::vector<float> dinv(N);
    for (int i = 0; i < N; ++i) dinv[i] = ptr[i + 1] > ptr[i] ? 1.f / (float)(ptr[i + 1] - ptr[i]) : 0.f;
    const int rc = alloc_graph(w, N, (int)adj.size());
    if (rc) return rc;
    GK(cudaMemcpyAsync(w->ptr.p, ptr.data(), sizeof(int) * ptr.size(), cudaMemcpyHostToDevice, st));
    if (!adj.empty()) {
        GK(cudaMemcpyAsync(w->adj.p, adj.data(), sizeof(int) * adj.size(), cudaMemcpyHostToDevice, st));
        GK(cudaMemcpyAsync(w->rev.p, rev.data(), sizeof(int) * rev.size(), cudaMemcpyHostToDevice, st));
    }
    GK(cudaMemcpyAsync(w->deg_inv.p, dinv.data(), sizeof(float) * N, cudaMemcpyHostToDevice, st));
    GK(cudaStreamSynchronize(st));
    return PDG_OK;
}

}  // namespace

// ---- solver-side hooks (declared in pdg_solver.h) -------------------------
namespace pdg {

int warm_infer_enqueue(pdg_warmstart* w, pdg_solver* s)
{
    cudaStream_t st = s->stream;
    const int N = w->N;
    k_node_feat<<<nb(N, 256), 256, 0, st>>>(N, s->X.p, s->V.p, s->Y.p, s->aux.p, w->stat.p, s->vcloth.p, s->cinfo.p,
                                            s->dprev.p, w->xin.p);
    k_edge_feat<<<nb(N, 256), 256, 0, st>>>(N, w->ptr.p, w->adj.p, w->rest.p, s->Y.p, w->ef.p);
    // encoder + layer 0's P, Q; per layer the messages, then the update fused
    // with the next layer's P, Q or, after the last layer, with the decoder
    // and the start offsets
    const Layout& y = w->lay;
    const float* p = w->p.p;
    fused<FUSE_ENC_PQ>(st, w->xin.p, NFP, N, w->W.We, p + y.be, w->W.AB[0], nullptr, w->cat[0].p, 2 * H, w->pq[0].p,
                       nullptr, nullptr, nullptr);
    for (int l = 0; l < L; ++l) {
        k_msg_fwd<<<msg_grid(N), 256, 0, st>>>(N, w->ptr.p, w->adj.p, w->ef.p, w->deg_inv.p, w->pq[l].p, p + y.C[l],
                                              p + y.c[l], w->cat[l].p);
        if (l + 1 < L)
            fused<FUSE_UPD_PQ>(st, w->cat[l].p, 2 * H, N, w->W.U[l], p + y.u[l], w->W.AB[l + 1], nullptr,
                               w->cat[l + 1].p, 2 * H, w->pq[l + 1].p, nullptr, nullptr, nullptr);
        else
            fused<FUSE_UPD_OUT>(st, w->cat[l].p, 2 * H, N, w->W.U[l], p + y.u[l], w->W.Wd, w->bdp.p, nullptr, 0,
                                nullptr, s->A.p, s->dprev.p, s->warm.p);
    }
    GK(cudaGetLastError());
    return PDG_OK;
}

// launches of one warm_infer_enqueue: features (2), encoder, per layer the
// messages and the fused update
int warm_kernel_count() { return 3 + 2 * L; }

void warm_detach(pdg_warmstart* w)
{
    if (w) w->solver = nullptr;
}

int warm_judge_sweeps(const pdg_warmstart* w) { return w ? w->judge : 0; }

}  // namespace pdg

extern "C" {

int pdg_warmstart_create(unsigned long long seed, pdg_warmstart** out)
{
    if (!out) return set_error(PDG_ERR_ARG, "pdg_warmstart_create: null output");
    std::unique_ptr<pdg_warmstart> w(new pdg_warmstart);
    GK(cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking));
    w->own_stream = true;
    int rc = alloc_params(w.get());
    if (rc) return rc;
    // uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights, zero biases; the
    // decoder starts at zero, so an untrained network predicts no change of
    // the offset: the previous frame's offset where it is valid, else y
    const Layout& y = w->lay;
    std::vector<float> h(y.total, 0.f);
    std::mt19937_64 rng(seed);
    auto fill = [&](int off, int rows, int cols, float gain) {
        std::uniform_real_distribution<float> U(-gain / std::sqrt((float)cols), gain / std::sqrt((float)cols));
        for (int i = 0; i < rows * cols; ++i) h[off + i] = U(rng);
    };
    fill(y.We, H, NF, 1.f);
    for (int l = 0; l < L; ++l) {
        fill(y.A[l], H, H, 1.f); fill(y.B[l], H, H, 1.f); fill(y.C[l], H, EF, 1.f); fill(y.U[l], H, 2 * H, 1.f);
    }
    // (decoder Wd, bd stay zero)
    GK(cudaMemcpyAsync(w->p.p, h.data(), sizeof(float) * y.total, cudaMemcpyHostToDevice, w->stream));
    rc = refresh_bf16(w.get(), w->stream);
    if (rc) return rc;
    GK(cudaStreamSynchronize(w->stream));
    *out = w.release();
    return PDG_OK;
}

int pdg_warmstart_param_count(const pdg_warmstart* w, int* n)
{
    if (!w || !n) return set_error(PDG_ERR_ARG, "null argument");
    *n = w->lay.total;
    return PDG_OK;
}

int pdg_warmstart_get_params(pdg_warmstart* w, float* host)
{
    if (!w || !host) return set_error(PDG_ERR_ARG, "null argument");
    GK(cudaStreamSynchronize(w->stream));
    if (w->solver) GK(cudaStreamSynchronize(w->solver->stream));
    GK(cudaMemcpyAsync(host, w->p.p, sizeof(float) * w->lay.total, cudaMemcpyDeviceToHost, w->stream));
    GK(cudaStreamSynchronize(w->stream));
    return PDG_OK;
}

int pdg_warmstart_set_params(pdg_warmstart* w, const float* host)
{
    if (!w || !host) return set_error(PDG_ERR_ARG, "null argument");
    for (int i = 0; i < w->lay.total; ++i)
        if (!std::isfinite(host[i])) return set_error(PDG_ERR_ARG, "non-finite parameter %d", i);
    GK(cudaStreamSynchronize(w->stream));
    if (w->solver) GK(cudaStreamSynchronize(w->solver->stream));
    GK(cudaMemcpyAsync(w->p.p, host, sizeof(float) * w->lay.total, cudaMemcpyHostToDevice, w->stream));
    GK(cudaMemsetAsync(w->m.p, 0, sizeof(float) * w->lay.total, w->stream));
    GK(cudaMemsetAsync(w->v.p, 0, sizeof(float) * w->lay.total, w->stream));
    w->t = 0;
    const int rc = refresh_bf16(w, w->stream);
    if (rc) return rc;
    GK(cudaStreamSynchronize(w->stream));
    return PDG_OK;
}

int pdg_warmstart_eval(pdg_warmstart* w, int N, const float* x, const int* ptr, const int* adj, const float* ef,
                       const float* target, const float* freew, const float* ew, float* out, float* loss,
                       float* grads)
{
    if (!w || N <= 0 || !x || !ptr || !target || !freew) return set_error(PDG_ERR_ARG, "pdg_warmstart_eval: bad arguments");
    if (w->solver) return set_error(PDG_ERR_STATE, "pdg_warmstart_eval: the network is attached to a solver");
    const int E = ptr[N];
    if (E < 0 || (E > 0 && (!adj || !ef))) return set_error(PDG_ERR_ARG, "pdg_warmstart_eval: bad adjacency");
    cudaStream_t st = w->stream;
    std::vector<int> hp(ptr, ptr + N + 1), ha(adj, adj + E);
    int rc = upload_graph(w, hp, ha, st);
    if (rc) return rc;
    std::vector<bf16> xb((size_t)N * NFP);
    for (int i = 0; i < N; ++i)
        for (int k = 0; k < NFP; ++k) xb[(size_t)i * NFP + k] = __float2bfloat16_rn(k < NF ? x[(size_t)i * NF + k] : 0.f);
    GK(cudaMemcpyAsync(w->xin.p, xb.data(), sizeof(bf16) * xb.size(), cudaMemcpyHostToDevice, st));
    if (E) GK(cudaMemcpyAsync(w->ef.p, ef, sizeof(float4) * E, cudaMemcpyHostToDevice, st));
    GK(cudaMemcpyAsync(w->target.p, target, sizeof(float) * 3 * N, cudaMemcpyHostToDevice, st));
    GK(cudaMemcpyAsync(w->freew.p, freew, sizeof(float) * N, cudaMemcpyHostToDevice, st));
    if (ew && E) GK(cudaMemcpyAsync(w->ew.p, ew, sizeof(float) * E, cudaMemcpyHostToDevice, st));
    double cnt = 0.0;
    for (int i = 0; i < N; ++i) cnt += freew[i] > 0.f ? 3.0 : 0.0;
    rc = forward(w, st);
    if (rc) return rc;
    rc = backward(w, (float)(1.0 / std::max(cnt, 1.0)), (ew && E) ? w->ew.p : nullptr, st);
    if (rc) return rc;
    std::vector<float> o((size_t)N * 16);
    double l = 0.0;
    GK(cudaMemcpyAsync(o.data(), w->out.p, sizeof(float) * o.size(), cudaMemcpyDeviceToHost, st));
    GK(cudaMemcpyAsync(&l, w->loss.p, sizeof(double), cudaMemcpyDeviceToHost, st));
    if (grads) GK(cudaMemcpyAsync(grads, w->g.p, sizeof(float) * w->lay.total, cudaMemcpyDeviceToHost, st));
    GK(cudaStreamSynchronize(st));
    if (out)
        for (int i = 0; i < N; ++i)
            for (int c = 0; c < NO; ++c) out[3 * i + c] = o[(size_t)i * 16 + c];
    if (loss) *loss = (float)l;
    return PDG_OK;
}

int pdg_warmstart_adam_step(pdg_warmstart* w, float lr)
{
    if (!w || !(lr > 0.f)) return set_error(PDG_ERR_ARG, "pdg_warmstart_adam_step: bad arguments");
    cudaStream_t st = w->solver ? w->solver->stream : w->stream;
    const int rc = adam_step(w, lr, st);
    if (rc) return rc;
    GK(cudaStreamSynchronize(st));
    return PDG_OK;
}

int pdg_warmstart_attach(pdg_warmstart* w, pdg_solver* s)
{
    if (!w || !s) return set_error(PDG_ERR_ARG, "pdg_warmstart_attach: null argument");
    if (s->kernel != PDG_KERNEL_GRAPH && s->kernel != PDG_KERNEL_STREAM)
        return set_error(PDG_ERR_STATE, "pdg_warmstart_attach: the solver must use the per-sweep (graph) kernels");
    const HostLayout& Lh = s->L;
    const int N = Lh.ntot;
    // mesh adjacency in the solver's (reordered) numbering, both directions
    std::vector<std::vector<std::pair<int, float>>> nbr(N);
    std::vector<float4> stat(N);
    std::vector<int> iperm(N);
    for (int g = 0; g < N; ++g) iperm[Lh.perm_global[g]] = g;   // batch caller index -> reordered
    int vbase = 0;
    for (const auto& c : s->cloths) {
        const Topology& t = *c.topo;
        const size_t nE = t.edges.size() / 4;
        for (size_t e = 0; e < nE; ++e) {
            const int a = iperm[vbase + t.edges[4 * e]], b = iperm[vbase + t.edges[4 * e + 1]];
            const float r = std::max(t.rest_len[e], 1e-12f);
            nbr[a].push_back({b, r});
            nbr[b].push_back({a, r});
        }
        double ks = 0.0, kb = 0.0;
        for (float k : c.cons.k_stretch) ks += k;
        for (float k : c.cons.bend_k) kb += k;
        ks = c.cons.k_stretch.empty() ? 1.0 : ks / c.cons.k_stretch.size();
        kb = c.cons.bend_k.empty() ? 1e-3 : kb / c.cons.bend_k.size();
        for (int i = 0; i < c.mesh->N; ++i) {
            const int gidx = iperm[vbase + i];
            const float m = std::max(c.mesh->mass[i], 1e-12f);
            stat[gidx] = make_float4((std::log(m) + 11.f) / 2.f, (float)((std::log(std::max(ks, 1e-6)) - 6.9) / 1.2),
                                     (float)((std::log(std::max(kb, 1e-9)) + 4.6) / 1.2), 0.f);
        }
        vbase += c.mesh->N;
    }
    std::vector<int> ptr(N + 1, 0), adj;
    std::vector<float> rest;
    for (int i = 0; i < N; ++i) {
        std::sort(nbr[i].begin(), nbr[i].end(), [](const std::pair<int, float>& a, const std::pair<int, float>& b) {
            return a.first < b.first;
        });
        for (auto& q : nbr[i]) { adj.push_back(q.first); rest.push_back(q.second); }
        ptr[i + 1] = (int)adj.size();
    }
    // Energy-norm weights of the loss's edge term: the PD system matrix
    // M + K approximated by M plus a graph Laplacian whose diagonal is K's
    // own (the Jacobi diagonal minus the mass), per unit mass: vertex i
    // spreads sigma_i = (D_i - m_i) / m_i evenly over its deg_i edges, and
    // an edge takes the mean of its two ends.  Pinned vertices contribute 0.
    std::vector<float> sig(N, 0.f), ew(adj.size(), 0.f);
    for (int i = 0; i < N; ++i) {
        const float4 a = Lh.aux[i];
        const float m = Lh.mass[i];
        const int deg = ptr[i + 1] - ptr[i];
        if (a.w > 0.f && m > 0.f && deg > 0) sig[i] = std::max(0.f, (1.f / (a.w * m) - 1.f) / (float)deg);
    }
    for (int i = 0; i < N; ++i)
        for (int e = ptr[i]; e < ptr[i + 1]; ++e) ew[e] = 0.5f * (sig[i] + sig[adj[e]]);
    cudaStream_t st = s->stream;
    int rc = upload_graph(w, ptr, adj, st);
    if (rc) return rc;
    if (!rest.empty()) GK(cudaMemcpyAsync(w->rest.p, rest.data(), sizeof(float) * rest.size(), cudaMemcpyHostToDevice, st));
    if (!ew.empty()) GK(cudaMemcpyAsync(w->ew.p, ew.data(), sizeof(float) * ew.size(), cudaMemcpyHostToDevice, st));
    GK(cudaMemcpyAsync(w->stat.p, stat.data(), sizeof(float4) * N, cudaMemcpyHostToDevice, st));
    GK(s->warm.alloc(N));
    GK(cudaMemsetAsync(s->warm.p, 0, sizeof(float4) * N, st));
    // the solver's learned-start state: previous offsets (none valid yet)
    // and the learned chain of the judge
    if (s->dprev.n != (size_t)N) GK(s->dprev.alloc(N));
    GK(cudaMemsetAsync(s->dprev.p, 0, sizeof(float4) * N, st));
    GK(s->A2.alloc(N)); GK(s->B2.alloc(N));
    GK(s->crt2.alloc(Lh.ncloth));
    GK(s->acc2.alloc((size_t)Lh.ncloth * s->acc_stride));
    GK(cudaMemsetAsync(s->acc2.p, 0, sizeof(double) * (size_t)Lh.ncloth * s->acc_stride, st));
    GK(cudaStreamSynchronize(st));
    w->solver = s;
    s->ws = w;
    if (s->graph) { cudaGraphExecDestroy(s->graph); s->graph = nullptr; }
    return PDG_OK;
}

int pdg_warmstart_train_frame(pdg_warmstart* w, pdg_solver* s, float lr, float* loss)
{
    if (!w || !s || w->solver != s) return set_error(PDG_ERR_STATE, "pdg_warmstart_train_frame: not attached to this solver");
    cudaStream_t st = s->stream;
    const int N = w->N;
    GK(cudaMemcpyAsync(w->Xn.p, s->X.p, sizeof(float4) * N, cudaMemcpyDeviceToDevice, st));
    GK(cudaMemcpyAsync(w->Vn.p, s->V.p, sizeof(float4) * N, cudaMemcpyDeviceToDevice, st));
    GK(cudaMemcpyAsync(w->Dn.p, s->dprev.p, sizeof(float4) * N, cudaMemcpyDeviceToDevice, st));
    int rc = pdg_solver_step(s, 1, nullptr);
    if (rc) return rc;
    // inputs from (x_n, v_n, y, d_prev), target (x* - y - d_prev)/s from the solve
    k_node_feat<<<nb(N, 256), 256, 0, st>>>(N, w->Xn.p, w->Vn.p, s->Y.p, s->aux.p, w->stat.p, s->vcloth.p, s->cinfo.p,
                                            w->Dn.p, w->xin.p);
    k_edge_feat<<<nb(N, 256), 256, 0, st>>>(N, w->ptr.p, w->adj.p, w->rest.p, s->Y.p, w->ef.p);
    k_target<<<nb(N, 256), 256, 0, st>>>(N, s->X.p, s->Y.p, s->aux.p, w->Dn.p, w->target.p, w->freew.p);
    int nfree = 0;
    for (const auto& a : s->L.aux) nfree += a.w >= 0.f ? 1 : 0;
    rc = forward(w, st);
    if (rc) return rc;
    rc = backward(w, 1.f / (float)std::max(1, 3 * nfree), w->energy ? w->ew.p : nullptr, st);
    if (rc) return rc;
    if (lr > 0.f) {
        rc = adam_step(w, lr, st);
        if (rc) return rc;
    }
    // features and target 3, forward 2 + 3L, loss and backward 7 + 11L,
    // Adam and the bf16 refresh 3 + 3L
    s->launches += 3 + (2 + 3 * L) + (7 + 11 * L) + (lr > 0.f ? 3 + 3 * L : 0);
    double l = 0.0;
    GK(cudaMemcpyAsync(&l, w->loss.p, sizeof(double), cudaMemcpyDeviceToHost, st));
    GK(cudaStreamSynchronize(st));
    if (loss) *loss = (float)l;
    return PDG_OK;
}

int pdg_warmstart_train_pair(pdg_warmstart* w, pdg_solver* traj, pdg_solver* deep, float lr, float* loss)
{
    if (!w || !traj || !deep || w->solver != traj)
        return set_error(PDG_ERR_STATE, "pdg_warmstart_train_pair: the network must be attached to `traj`");
    if (deep == traj || deep->L.ntot != traj->L.ntot || deep->L.ncloth != traj->L.ncloth ||
        deep->L.perm_global != traj->L.perm_global || deep->kernel == PDG_KERNEL_PERSISTENT ||
        deep->kernel == PDG_KERNEL_RESIDENT)
        return set_error(PDG_ERR_ARG, "pdg_warmstart_train_pair: `deep` must solve the same cloths with the same "
                                      "vertex layout (same patch plan, per-sweep kernels)");
    cudaStream_t st = traj->stream;
    const int N = w->N;
    GK(cudaStreamSynchronize(deep->stream));
    // inputs (x_n, v_n, d_prev) of the trajectory; the deep solve starts from the same state
    GK(cudaMemcpyAsync(w->Xn.p, traj->X.p, sizeof(float4) * N, cudaMemcpyDeviceToDevice, st));
    GK(cudaMemcpyAsync(w->Vn.p, traj->V.p, sizeof(float4) * N, cudaMemcpyDeviceToDevice, st));
    GK(cudaMemcpyAsync(w->Dn.p, traj->dprev.p, sizeof(float4) * N, cudaMemcpyDeviceToDevice, st));
    GK(cudaMemcpyAsync(deep->X.p, traj->X.p, sizeof(float4) * N, cudaMemcpyDeviceToDevice, st));
    GK(cudaMemcpyAsync(deep->V.p, traj->V.p, sizeof(float4) * N, cudaMemcpyDeviceToDevice, st));
    GK(cudaStreamSynchronize(st));
    int rc = pdg_solver_step(deep, 1, nullptr);   // the target: x* of this frame
    if (rc) return rc;
    GK(cudaStreamSynchronize(deep->stream));
    rc = pdg_solver_step(traj, 1, nullptr);       // the trajectory and its kept offsets advance
    if (rc) return rc;
    // y of both solvers is the same prediction from the same state
    k_node_feat<<<nb(N, 256), 256, 0, st>>>(N, w->Xn.p, w->Vn.p, traj->Y.p, traj->aux.p, w->stat.p, traj->vcloth.p,
                                            traj->cinfo.p, w->Dn.p, w->xin.p);
    k_edge_feat<<<nb(N, 256), 256, 0, st>>>(N, w->ptr.p, w->adj.p, w->rest.p, traj->Y.p, w->ef.p);
    k_target<<<nb(N, 256), 256, 0, st>>>(N, deep->X.p, traj->Y.p, traj->aux.p, w->Dn.p, w->target.p, w->freew.p);
    int nfree = 0;
    for (const auto& a : traj->L.aux) nfree += a.w >= 0.f ? 1 : 0;
    rc = forward(w, st);
    if (rc) return rc;
    rc = backward(w, 1.f / (float)std::max(1, 3 * nfree), w->energy ? w->ew.p : nullptr, st);
    if (rc) return rc;
    if (lr > 0.f) {
        rc = adam_step(w, lr, st);
        if (rc) return rc;
    }
    traj->launches += 3 + (2 + 3 * L) + (7 + 11 * L) + (lr > 0.f ? 3 + 3 * L : 0);
    double l = 0.0;
    GK(cudaMemcpyAsync(&l, w->loss.p, sizeof(double), cudaMemcpyDeviceToHost, st));
    GK(cudaStreamSynchronize(st));
    if (loss) *loss = (float)l;
    return PDG_OK;
}

int pdg_warmstart_set_smoothness(pdg_warmstart* w, float lambda)
{
    if (!w || !(lambda >= 0.f) || !std::isfinite(lambda))
        return set_error(PDG_ERR_ARG, "pdg_warmstart_set_smoothness: lambda must be finite and >= 0");
    w->smooth = lambda;
    return PDG_OK;
}

int pdg_warmstart_time_inference(pdg_warmstart* w, int reps, float* ms)
{
    if (!w || reps <= 0 || !ms) return set_error(PDG_ERR_ARG, "pdg_warmstart_time_inference: bad arguments");
    pdg_solver* s = w->solver;
    if (!s) return set_error(PDG_ERR_STATE, "pdg_warmstart_time_inference: not attached to a solver");
    cudaEvent_t e0, e1;
    GK(cudaEventCreate(&e0));
    GK(cudaEventCreate(&e1));
    int rc = warm_infer_enqueue(w, s);   // untimed first run
    GK(cudaEventRecord(e0, s->stream));
    for (int r = 0; r < reps && rc == PDG_OK; ++r) rc = warm_infer_enqueue(w, s);
    GK(cudaEventRecord(e1, s->stream));
    GK(cudaEventSynchronize(e1));
    float t = 0.f;
    GK(cudaEventElapsedTime(&t, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    s->launches += (long long)(reps + 1) * warm_kernel_count();
    *ms = t / (float)reps;
    return PDG_OK;
}

int pdg_warmstart_set_energy_norm(pdg_warmstart* w, int enable)
{
    if (!w) return set_error(PDG_ERR_ARG, "pdg_warmstart_set_energy_norm: null argument");
    w->energy = enable ? 1 : 0;
    return PDG_OK;
}

int pdg_warmstart_set_judge_sweeps(pdg_warmstart* w, int sweeps)
{
    if (!w || sweeps < 0 || sweeps > 1000)
        return set_error(PDG_ERR_ARG, "pdg_warmstart_set_judge_sweeps: sweeps must be in [0, 1000]");
    w->judge = sweeps;
    // the frame graph of an attached solver holds the judge's launches
    if (w->solver && w->solver->graph) { cudaGraphExecDestroy(w->solver->graph); w->solver->graph = nullptr; }
    return PDG_OK;
}

int pdg_warmstart_get_judge_sweeps(const pdg_warmstart* w, int* sweeps)
{
    if (!w || !sweeps) return set_error(PDG_ERR_ARG, "pdg_warmstart_get_judge_sweeps: null argument");
    *sweeps = w->judge;
    return PDG_OK;
}

void pdg_warmstart_destroy(pdg_warmstart* w)
{
    if (!w) return;
    if (w->solver) { w->solver->ws = nullptr; if (w->solver->graph) { cudaGraphExecDestroy(w->solver->graph); w->solver->graph = nullptr; } }
    delete w;
}

}  // extern "C"
