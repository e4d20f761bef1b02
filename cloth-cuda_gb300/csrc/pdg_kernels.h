// Host-callable launchers of the PD kernels (implemented in *.cu files).
#pragma once

#include <cuda_runtime.h>

#include "pdg_layout.h"

namespace pdg {

cudaError_t launch_iter(const IterArgs& a, int mode, int nt, int npatch, size_t smem, int k, int res_only,
                        cudaStream_t s, int carveout = 0);
cudaError_t launch_predict(const IterArgs& a, const float4* X, const float4* V, const float4* aux,
                           const float* mass, const int* vcloth, const float4* warm, int n, cudaStream_t s);
cudaError_t launch_finalize(const IterArgs& a, float4* X, float4* V, const float4* aux, const int* vcloth, int n,
                            cudaStream_t s);
// Residuals of the inertial start (buf[0]) and of the learned start `warm`,
// then the per-cloth choice between them (slots acc_stride-2 / -1).
cudaError_t launch_warm_select(const IterArgs& a, int nt, int npatch, size_t smem, const float4* warm,
                               const int* vcloth, int n, cudaStream_t s);
// Learned start judged after K sweeps: r(y) of the inertial start (with
// `eval_start`; else launch_warm_start_norm takes it from the inertial
// chain's first sweep), then the start records and iterates of the inertial
// chain `a` and the learned chain `b` (same layout, own iterates, records and
// per-sweep sums).
cudaError_t launch_warm_chain_init(const IterArgs& a, const IterArgs& b, int nt, int npatch, size_t smem,
                                   const float4* warm, const int* vcloth, int n, bool eval_start, cudaStream_t s);
// Both chains' normaliser r(y)^2 from the inertial chain's sweep-0 residual
// sum (between its sweeps 0 and 1).
cudaError_t launch_warm_start_norm(const IterArgs& a, const IterArgs& b, cudaStream_t s);
// After K sweeps of both chains: per cloth the chain with the lower residual
// continues on `a`.
cudaError_t launch_warm_judge(const IterArgs& a, const IterArgs& b, int K, const int* vcloth, int n, cudaStream_t s);
// After a frame: each vertex's offset x - y into dprev (w = 1 valid), the
// learned start's previous-offset feature of the next frame.
cudaError_t launch_keep_offset(const IterArgs& a, const float4* X, const float4* aux, const int* vcloth, float4* dprev,
                               int n, cudaStream_t s);
// Caller order <-> solver order for one array, or two in one launch (src1/dst1).
// dprev (may be null): vertices whose state changes lose their kept
// previous-frame offset (the learned start's feature).
cudaError_t launch_scatter_state(const float* src, float4* dst, const int* perm, int n, cudaStream_t s,
                                 const float* src1 = nullptr, float4* dst1 = nullptr, float4* dprev = nullptr);
cudaError_t launch_gather_state(const float4* src, float* dst, const int* perm, int n, cudaStream_t s,
                                const float4* src1 = nullptr, float* dst1 = nullptr);
// Whole-batch copies in caller order (inv: caller index -> reordered vertex);
// x / v may be device pointers or mapped page-locked host memory.
cudaError_t launch_put_state(const float* x, const float* v, float4* X, float4* V, const int* inv, int n,
                             cudaStream_t s, float4* dprev = nullptr);
cudaError_t launch_take_state(const float4* X, const float4* V, float* x, float* v, const int* inv, int n,
                              cudaStream_t s);
cudaError_t launch_apply_pins(float* pos, float* vel, const int* idx, const float* target, int P,
                              cudaStream_t s);

// Persistent whole-frame kernel (pd_persistent.cu).
struct PersistArgs {
    IterArgs it;
    const float4* X;
    float4* Xw;          // state x (written at the end of the frame)
    float4* V;
    const float4* aux;
    const float* mass;
    const int* vcloth;
    const float4* warm;
    float4* Y;
    int n;               // vertices
    int npatch;
    int max_iter;        // largest cap over cloths
    int have_final;      // evaluate r(x) of the returned iterate
    int mode;
    unsigned* bar;       // [0] arrive counter, [1] generation
    int* err;            // set when a grid barrier times out
    long long spin_budget;  // clock64 cycles a barrier may wait
    // neighbour synchronisation of the resident kernel (fixed sweep counts):
    // the boundary offsets d^k of every vertex as tagged words, buffer k & 1
    // at xch[((k & 1) * n + vertex) * 4 + component], each word the value's
    // bits | (tag0 + k) << 32.  tag0 is read from the device word *xch_tag,
    // which every frame advances by its sweep count (null: no exchange)
    unsigned long long* xch;
    unsigned* xch_tag;
    int nbr_sync;        // 1: sweeps wait for neighbour patches only
    // caller state moved inside the frame launch (resident kernel only): x, v
    // read by the prediction and written by the finalisation, AoS xyz in
    // caller order; any may be null.  Device or page-locked mapped host
    // memory.  With caller arrays the prediction and the finalisation walk
    // the vertices in caller order (io_inv: caller vertex -> layout vertex),
    // so that host memory is read and written contiguously.
    const float* in_x;
    const float* in_v;
    float* out_x;
    float* out_v;
    const int* io_inv;
};
cudaError_t launch_persistent(const PersistArgs& p, int nt, int grid, size_t smem, cudaStream_t s);
int persistent_max_blocks(int mode, int nt, size_t smem, int* per_sm);

// Resident persistent kernel (pd_resident.cu): one patch per block for the
// whole frame; nt compute threads (480: one block per SM, 224: two) plus one
// warp.  Limit: nown <= nt.  Kernel variant for nt threads (-1: none).
int resident_pick(int nt);
int resident_max_blocks(int mode, int variant, size_t smem);
// Whether the kernel has an instance that moves the caller's state (PersistArgs
// in_x ... out_v) for this mode.
bool resident_moves_state(int mode);
cudaError_t launch_resident(const PersistArgs& p, int variant, int grid, size_t smem, cudaStream_t s);

// Streaming per-sweep kernel (pd_stream.cu): persistent grid, the vertex
// data of each block's next patch double-buffered in shared memory by bulk
// and asynchronous copies.  Byte offsets of the regions of one stage; the
// vertex-major contribution slots follow the two stages.
struct StreamArgs {
    int o_hidx, o_ptr, o_y, o_d, o_dp;
    int stage_bytes;
    int slot_off;
    int max_nslot;          // vertex-major slots per patch (largest)
    int npatch;
    int* err;               // set when a copy wait times out
    long long spin_budget;  // clock64 cycles a wait may take
};
bool stream_layout(int max_nown, int max_nhalo, int max_nlocal, int max_vm_nslot, StreamArgs& sa, size_t& smem);
int stream_max_blocks(int mode, int nt, size_t smem);
// after_sweep: the previous launch on the stream is a sweep of this kernel;
// the launch then overlaps its tail (programmatic dependent launch).
cudaError_t launch_stream(const IterArgs& a, const StreamArgs& sa, int mode, int nt, int grid, size_t smem, int k,
                          int res_only, cudaStream_t s, bool after_sweep);

}  // namespace pdg
