// Learned warm start for the PD solve (no counterpart in the reference).
//
// A 2-layer mesh message-passing network (hidden 64) predicts, per vertex,
// the offset d = x* - y of the converged position from the inertial
// prediction.  Node GEMMs run on the tensor cores (bf16 mma.sync m16n8k16,
// fp32 accumulation, bf16 activations); edge messages are warp-per-node
// gathers over the mesh adjacency (deterministic, no atomics); weight
// gradients are fp32 per-block partial sums added in a fixed block order
// (bitwise reproducible); Adam keeps fp32 master weights and refreshes their
// bf16 copies after each step.
//
// Network (x: 14 node features, e_ij: 4 edge features):
//   h0 = relu(We x + be)
//   per layer: P = A h, Q = B h;  m_ij = relu(P_i + Q_j + C e_ij + c);
//              a_i = mean_j m_ij;  h <- h + relu(U [h; a] + u)
//   out = Wd h + bd     ((offset - previous offset) / kOffsetScale)
#include "gnn.cuh"
#include "pdg_solver.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

namespace pdg {
namespace gnn {

using bf16 = __nv_bfloat16;

enum { EPI_RELU = 1, EPI_STORE1 = 2, EPI_RESID2 = 4, EPI_STOREF = 8, EPI_ACCF = 16, EPI_RESIDA = 32 };

__device__ __forceinline__ uint32_t ld_pair(const bf16* p) { return *reinterpret_cast<const uint32_t*>(p); }
__device__ __forceinline__ uint32_t ld_pair(const float* p)
{
    const float2 f = *reinterpret_cast<const float2*>(p);
    __nv_bfloat162 b = __floats2bfloat162_rn(f.x, f.y);
    return *reinterpret_cast<uint32_t*>(&b);
}

__device__ __forceinline__ void mma_bf16(float* c, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Y[M x NOUT] = X[M x K] W^T (+ bias), W stored [NOUT][K] bf16.  A block
// stages W (with a padded row stride of K + 8 elements, so the B-fragment
// loads are bank-conflict free) and the bias in shared memory once, in
// 16-byte pieces, and its warps then walk 16-row tiles with a grid stride
// (gemm_grid sizes the grid to the resident blocks).
// Epilogue: optional ReLU; Y1 <- bf16(v); Y2 <- bf16(R + v) (R read, or taken
// from the A fragments when it is X's first NOUT columns); Yf <- v or += v.
template <typename TA, int K, int NOUT, int EPI>
__global__ void __launch_bounds__(128) k_gemm(const TA* __restrict__ X, int ldx, int M, const bf16* __restrict__ W,
                                              const float* __restrict__ bias, const bf16* __restrict__ R, int ldr,
                                              bf16* __restrict__ Y1, int ld1, bf16* __restrict__ Y2, int ld2,
                                              float* __restrict__ Yf, int ldf)
{
    static_assert(K % 16 == 0 && NOUT % 8 == 0, "mma tile shape");
    static_assert(!(EPI & EPI_RESIDA) || NOUT <= K, "the residual is part of the A operand");
    __shared__ __align__(16) bf16 sW[NOUT * (K + 8)];
    __shared__ float sb[NOUT];
    for (int i = threadIdx.x; i < NOUT * K / 8; i += 128) {
        const int r = i / (K / 8), c = (i % (K / 8)) * 8;
        *reinterpret_cast<uint4*>(sW + r * (K + 8) + c) = *reinterpret_cast<const uint4*>(W + (size_t)r * K + c);
    }
    for (int i = threadIdx.x; i < NOUT; i += 128) sb[i] = bias ? bias[i] : 0.f;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int ntile = (M + 15) >> 4, stride = gridDim.x * 4;
    // A fragments of row tile `tl` (zero rows past M)
    auto load_a = [&](int tl, uint32_t (&f)[K / 16][4]) {
        const int r0 = tl * 16;
        const bool ok0 = r0 + g < M, ok1 = r0 + g + 8 < M;
        const TA* x0 = X + (size_t)(r0 + g) * ldx;
        const TA* x1 = X + (size_t)(r0 + g + 8) * ldx;
        #pragma unroll
        for (int ks = 0; ks < K / 16; ++ks) {
            const int c0 = ks * 16 + 2 * t;
            f[ks][0] = ok0 ? ld_pair(x0 + c0) : 0u;
            f[ks][1] = ok1 ? ld_pair(x1 + c0) : 0u;
            f[ks][2] = ok0 ? ld_pair(x0 + c0 + 8) : 0u;
            f[ks][3] = ok1 ? ld_pair(x1 + c0 + 8) : 0u;
        }
    };
    int tile = blockIdx.x * 4 + warp;
    uint32_t a[K / 16][4];
    load_a(tile, a);
    for (; tile < ntile; tile += stride) {
        const int r0 = tile * 16;
        // the next tile's fragments are loaded while this one is multiplied
        uint32_t an[K / 16][4];
        load_a(tile + stride, an);
        float acc[NOUT / 8][4];
        #pragma unroll
        for (int n = 0; n < NOUT / 8; ++n) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.f;
        #pragma unroll
        for (int ks = 0; ks < K / 16; ++ks) {
            const int c0 = ks * 16 + 2 * t;
            #pragma unroll
            for (int n = 0; n < NOUT / 8; ++n) {
                const bf16* wr = sW + (n * 8 + g) * (K + 8) + c0;
                mma_bf16(acc[n], a[ks][0], a[ks][1], a[ks][2], a[ks][3], *reinterpret_cast<const uint32_t*>(wr),
                         *reinterpret_cast<const uint32_t*>(wr + 8));
            }
        }
        #pragma unroll
        for (int n = 0; n < NOUT / 8; ++n)
            #pragma unroll
            for (int hf = 0; hf < 2; ++hf) {
                const int row = r0 + g + 8 * hf;
                if (row >= M) continue;
                const int col = n * 8 + 2 * t;
                float v0 = acc[n][2 * hf], v1 = acc[n][2 * hf + 1];
                if (bias) { v0 += sb[col]; v1 += sb[col + 1]; }
                if (EPI & EPI_RELU) { v0 = fmaxf(v0, 0.f); v1 = fmaxf(v1, 0.f); }
                if (EPI & EPI_STORE1)
                    *reinterpret_cast<__nv_bfloat162*>(Y1 + (size_t)row * ld1 + col) = __floats2bfloat162_rn(v0, v1);
                if (EPI & (EPI_RESID2 | EPI_RESIDA)) {
                    // EPI_RESIDA: the residual is the A operand's first NOUT
                    // columns, already in this thread's fragments
                    __nv_bfloat162 r;
                    if (EPI & EPI_RESIDA) {
                        const uint32_t u = a[n >> 1][(n & 1) * 2 + hf];
                        r = *reinterpret_cast<const __nv_bfloat162*>(&u);
                    } else {
                        r = *reinterpret_cast<const __nv_bfloat162*>(R + (size_t)row * ldr + col);
                    }
                    *reinterpret_cast<__nv_bfloat162*>(Y2 + (size_t)row * ld2 + col) =
                        __floats2bfloat162_rn(__bfloat162float(r.x) + v0, __bfloat162float(r.y) + v1);
                }
                if (EPI & EPI_STOREF) *reinterpret_cast<float2*>(Yf + (size_t)row * ldf + col) = make_float2(v0, v1);
                if (EPI & EPI_ACCF) {
                    float2* p = reinterpret_cast<float2*>(Yf + (size_t)row * ldf + col);
                    const float2 o = *p;
                    *p = make_float2(o.x + v0, o.y + v1);
                }
            }
        #pragma unroll
        for (int ks = 0; ks < K / 16; ++ks)
            #pragma unroll
            for (int i = 0; i < 4; ++i) a[ks][i] = an[ks][i];
    }
}

// Grid of a grid-stride kernel: `need` blocks, at most the blocks of
// `threads` threads and `smem` dynamic shared bytes that are resident at once
// on the current device (looked up once per kernel and device; the kernel's
// dynamic shared-memory limit is raised to `smem` then).
template <auto KERN>
int resident_grid(int threads, size_t smem, long long need)
{
    static int resident[16] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    int& r = resident[dev & 15];
    if (r == 0) {
        int nsm = 0, per = 0;
        if (smem > 48 * 1024) cudaFuncSetAttribute(KERN, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, KERN, threads, smem);
        r = std::max(1, nsm * std::max(per, 1));
    }
    return (int)std::max(1LL, std::min(need, (long long)r));
}

// Grid of k_gemm for M rows: enough blocks for every row tile, at most the
// resident ones.
template <typename TA, int K, int NOUT, int EPI>
int gemm_grid(int M)
{
    return resident_grid<k_gemm<TA, K, NOUT, EPI>>(128, 0, ((((long long)M + 15) >> 4) + 3) / 4);
}

// Launch of k_gemm on `st` with the grid above.
template <typename TA, int K, int NOUT, int EPI>
void gemm(cudaStream_t st, const TA* X, int ldx, int M, const bf16* W, const float* bias, const bf16* R, int ldr,
          bf16* Y1, int ld1, bf16* Y2, int ld2, float* Yf, int ldf)
{
    k_gemm<TA, K, NOUT, EPI><<<gemm_grid<TA, K, NOUT, EPI>(M), 128, 0, st>>>(X, ldx, M, W, bias, R, ldr, Y1, ld1, Y2,
                                                                            ld2, Yf, ldf);
}

// ---- fused inference kernels ----------------------------------------------
// One warp holds a 16-row tile from its first product to its last store: the
// first product's epilogue rounds h to bf16 in the accumulator layout of
// m16n8k16, which is exactly the A-fragment layout of the next mma (n-tiles
// 2k and 2k+1 form k-step k), so the second product starts from registers.
// Every product is the mma sequence k_gemm issues on the same bf16 operands
// and every epilogue the same float operations, so the results are bitwise
// those of the separate kernels (encoder; update; P/Q; decoder + start).
//   FUSE_ENC_PQ:  h = relu(We x + be), stored; P, Q = AB h of layer 0
//   FUSE_UPD_PQ:  h' = h + relu(U [h; a] + u), stored; P, Q = AB h' of the next layer
//   FUSE_UPD_OUT: h' as above; out = Wd h' + bd; warm start d_prev + s out
// B fragments come from the staged weights by ldmatrix (two n-tiles per
// instruction); outputs go through a per-warp shared tile (stmatrix) and
// leave as 16-byte row pieces.
enum { FUSE_ENC_PQ = 0, FUSE_UPD_PQ = 1, FUSE_UPD_OUT = 2 };

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void ldsm_x4(const bf16* p, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(smem_u32(p)));
}
__device__ __forceinline__ void stsm_x4(bf16* p, uint32_t r0, uint32_t r1, uint32_t r2, uint32_t r3)
{
    asm volatile("stmatrix.sync.aligned.m8n8.x4.shared.b16 [%0], {%1,%2,%3,%4};" ::"r"(smem_u32(p)), "r"(r0), "r"(r1),
                 "r"(r2), "r"(r3)
                 : "memory");
}

// acc[n] (n-tiles 0..NT-1) += A (16 x K, fragments a) W^T, W staged as
// [NT*8][K + 8]: one ldmatrix.x4 gives b0, b1 of n-tiles n and n + 1.
template <int K, int NT>
__device__ __forceinline__ void mma_tile(float (&acc)[NT][4], const uint32_t (&a)[K / 16][4], const bf16* sW,
                                         int lane)
{
    const int m = lane >> 3, r = lane & 7;
    #pragma unroll
    for (int ks = 0; ks < K / 16; ++ks)
        #pragma unroll
        for (int n = 0; n < NT; n += 2) {
            uint32_t b00, b01, b10, b11;
            ldsm_x4(sW + ((n + (m >> 1)) * 8 + r) * (K + 8) + ks * 16 + (m & 1) * 8, b00, b01, b10, b11);
            mma_bf16(acc[n], a[ks][0], a[ks][1], a[ks][2], a[ks][3], b00, b01);
            mma_bf16(acc[n + 1], a[ks][0], a[ks][1], a[ks][2], a[ks][3], b10, b11);
        }
}

// Rows r0..r0+15 of a bf16 tile (the first COLS columns of sO, row stride
// SROW) to global memory (row stride ld), 16 bytes per piece.
template <int COLS, int SROW>
__device__ __forceinline__ void tile_out(const bf16* sO, bf16* dst, int ld, int r0, int M, int lane)
{
    constexpr int PR = COLS / 8;   // 16-byte pieces per row
    #pragma unroll
    for (int q = lane; q < 16 * PR; q += 32) {
        const int row = q / PR, c = (q % PR) * 8;
        if (r0 + row < M)
            *reinterpret_cast<uint4*>(dst + (size_t)(r0 + row) * ld + c) =
                *reinterpret_cast<const uint4*>(sO + row * SROW + c);
    }
}

// Fragment pairs c[n][0..1] (rows 0-7 / 8-15 of n-tile n, bf16x2) of NT
// n-tiles into the staged tile sO (row stride COLS + 8) at column col0.
template <int NT, int COLS>
__device__ __forceinline__ void tile_stage(const uint32_t (&c)[NT][2], bf16* sO, int col0, int lane)
{
    const int m = lane >> 3, r = lane & 7;
    #pragma unroll
    for (int n = 0; n < NT; n += 2)
        stsm_x4(sO + ((m & 1) * 8 + r) * (COLS + 8) + col0 + (n + (m >> 1)) * 8, c[n][0], c[n][1], c[n + 1][0],
                c[n + 1][1]);
}

template <int MODE>
struct FusedShape {
    static constexpr int K1 = MODE == FUSE_ENC_PQ ? NFP : 2 * H;   // first product: K1 -> H
    static constexpr int N2 = MODE == FUSE_UPD_OUT ? 8 : 2 * H;     // second: H -> N2 (decoder: first n-tile)
    static constexpr int OCOLS = MODE == FUSE_UPD_OUT ? 8 : 2 * H;  // staged output tile width
    static constexpr size_t smem = sizeof(bf16) * ((size_t)H * (K1 + 8) + (size_t)N2 * (H + 8) +
                                                   (MODE == FUSE_UPD_OUT ? 0 : 4 * 16 * (OCOLS + 8)));
};

template <int MODE>
__global__ void __launch_bounds__(128, 4) k_fused(const bf16* __restrict__ X, int ldx, int M,
                                                  const bf16* __restrict__ W1, const float* __restrict__ b1,
                                                  const bf16* __restrict__ W2, const float* __restrict__ b2,
                                                  bf16* __restrict__ hout, int ldh, bf16* __restrict__ pq,
                                                  const float4* __restrict__ A, const float4* __restrict__ Dp,
                                                  float4* __restrict__ warm)
{
    using S = FusedShape<MODE>;
    constexpr int K1 = S::K1, N2 = S::N2;
    extern __shared__ __align__(16) unsigned char fsm[];
    bf16* sW1 = reinterpret_cast<bf16*>(fsm);
    bf16* sW2 = sW1 + H * (K1 + 8);
    __shared__ float sb1[H], sb2[N2];
    for (int i = threadIdx.x; i < H * K1 / 8; i += 128) {
        const int r = i / (K1 / 8), c = (i % (K1 / 8)) * 8;
        *reinterpret_cast<uint4*>(sW1 + r * (K1 + 8) + c) = *reinterpret_cast<const uint4*>(W1 + (size_t)r * K1 + c);
    }
    for (int i = threadIdx.x; i < N2 * H / 8; i += 128) {
        const int r = i / (H / 8), c = (i % (H / 8)) * 8;
        *reinterpret_cast<uint4*>(sW2 + r * (H + 8) + c) = *reinterpret_cast<const uint4*>(W2 + (size_t)r * H + c);
    }
    for (int i = threadIdx.x; i < H; i += 128) sb1[i] = b1[i];
    for (int i = threadIdx.x; i < N2; i += 128) sb2[i] = b2 ? b2[i] : 0.f;
    __syncthreads();
    const unsigned full = 0xffffffffu;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    bf16* sO = sW2 + N2 * (H + 8) + warp * 16 * (S::OCOLS + 8);   // this warp's output tile
    const int ntile = (M + 15) >> 4, stride = gridDim.x * 4;
    auto load_a = [&](int tl, uint32_t (&f)[K1 / 16][4]) {
        const int r0 = tl * 16;
        const bool ok0 = r0 + g < M, ok1 = r0 + g + 8 < M;
        const bf16* x0 = X + (size_t)(r0 + g) * ldx;
        const bf16* x1 = X + (size_t)(r0 + g + 8) * ldx;
        #pragma unroll
        for (int ks = 0; ks < K1 / 16; ++ks) {
            const int c0 = ks * 16 + 2 * t;
            f[ks][0] = ok0 ? ld_pair(x0 + c0) : 0u;
            f[ks][1] = ok1 ? ld_pair(x1 + c0) : 0u;
            f[ks][2] = ok0 ? ld_pair(x0 + c0 + 8) : 0u;
            f[ks][3] = ok1 ? ld_pair(x1 + c0 + 8) : 0u;
        }
    };
    int tile = blockIdx.x * 4 + warp;
    uint32_t a[K1 / 16][4];
    load_a(tile, a);
    for (; tile < ntile; tile += stride) {
        const int r0 = tile * 16;
        uint32_t an[K1 / 16][4];
        load_a(tile + stride, an);
        // first product and its epilogue: hp = bf16(h) in fragment layout
        uint32_t hp[H / 8][2];
        {
            float acc[H / 8][4];
            #pragma unroll
            for (int n = 0; n < H / 8; ++n) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.f;
            mma_tile<K1, H / 8>(acc, a, sW1, lane);
            #pragma unroll
            for (int n = 0; n < H / 8; ++n)
                #pragma unroll
                for (int hf = 0; hf < 2; ++hf) {
                    const int col = n * 8 + 2 * t;
                    const float v0 = fmaxf(acc[n][2 * hf] + sb1[col], 0.f);
                    const float v1 = fmaxf(acc[n][2 * hf + 1] + sb1[col + 1], 0.f);
                    __nv_bfloat162 o;
                    if (MODE == FUSE_ENC_PQ) {
                        o = __floats2bfloat162_rn(v0, v1);
                    } else {   // residual: the A operand's first H columns
                        const uint32_t u = a[n >> 1][(n & 1) * 2 + hf];
                        const __nv_bfloat162 r = *reinterpret_cast<const __nv_bfloat162*>(&u);
                        o = __floats2bfloat162_rn(__bfloat162float(r.x) + v0, __bfloat162float(r.y) + v1);
                    }
                    hp[n][hf] = *reinterpret_cast<const uint32_t*>(&o);
                }
        }
        if (MODE != FUSE_UPD_OUT) {
            constexpr int OC = S::OCOLS;
            tile_stage<H / 8, OC>(hp, sO, 0, lane);
            __syncwarp();
            tile_out<H, OC + 8>(sO, hout, ldh, r0, M, lane);
            __syncwarp();
            // P, Q of the next layer, 64 columns at a time, staged then stored
            #pragma unroll
            for (int half = 0; half < 2; ++half) {
                float acc[8][4];
                #pragma unroll
                for (int n = 0; n < 8; ++n) acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.f;
                uint32_t hk[H / 16][4];
                #pragma unroll
                for (int ks = 0; ks < H / 16; ++ks) {
                    hk[ks][0] = hp[2 * ks][0]; hk[ks][1] = hp[2 * ks][1];
                    hk[ks][2] = hp[2 * ks + 1][0]; hk[ks][3] = hp[2 * ks + 1][1];
                }
                mma_tile<H, 8>(acc, hk, sW2 + half * H * (H + 8), lane);
                uint32_t c[8][2];
                #pragma unroll
                for (int n = 0; n < 8; ++n)
                    #pragma unroll
                    for (int hf = 0; hf < 2; ++hf) {
                        const __nv_bfloat162 o = __floats2bfloat162_rn(acc[n][2 * hf], acc[n][2 * hf + 1]);
                        c[n][hf] = *reinterpret_cast<const uint32_t*>(&o);
                    }
                tile_stage<8, OC>(c, sO, half * H, lane);
            }
            __syncwarp();
            tile_out<2 * H, OC + 8>(sO, pq, 2 * H, r0, M, lane);
            __syncwarp();
        } else {
            // decoder, first n-tile (outputs 0..7 of which 0..2 are used),
            // then the start offsets of the separate path
            float acc[4] = {0.f, 0.f, 0.f, 0.f};
            #pragma unroll
            for (int ks = 0; ks < H / 16; ++ks) {
                const int c0 = ks * 16 + 2 * t;
                const bf16* wr = sW2 + g * (H + 8) + c0;
                mma_bf16(acc, hp[2 * ks][0], hp[2 * ks][1], hp[2 * ks + 1][0], hp[2 * ks + 1][1],
                         *reinterpret_cast<const uint32_t*>(wr), *reinterpret_cast<const uint32_t*>(wr + 8));
            }
            #pragma unroll
            for (int hf = 0; hf < 2; ++hf) {
                // lane t holds outputs 2t, 2t+1 of rows g and g + 8; output 2
                // comes from the next lane (t = 1)
                const float o0 = acc[2 * hf] + sb2[2 * t], o1 = acc[2 * hf + 1] + sb2[2 * t + 1];
                const float o2 = __shfl_down_sync(full, o0, 1);
                const int row = r0 + g + 8 * hf;
                if (t == 0 && row < M) {
                    const float4 av = A[row];
                    const float4 dp = Dp ? Dp[row] : make_float4(0.f, 0.f, 0.f, 0.f);
                    const float ok = dp.w > 0.f ? 1.f : 0.f;
                    warm[row] = av.w < 0.f ? av
                                           : make_float4(fmaf(o0, kOffsetScale, ok * dp.x),
                                                         fmaf(o1, kOffsetScale, ok * dp.y),
                                                         fmaf(o2, kOffsetScale, ok * dp.z), av.w);
                }
            }
        }
        #pragma unroll
        for (int ks = 0; ks < K1 / 16; ++ks)
            #pragma unroll
            for (int i = 0; i < 4; ++i) a[ks][i] = an[ks][i];
    }
}

// Launch of k_fused on `st`, the grid sized to the resident blocks.
template <int MODE>
void fused(cudaStream_t st, const bf16* X, int ldx, int M, const bf16* W1, const float* b1, const bf16* W2,
           const float* b2, bf16* hout, int ldh, bf16* pq, const float4* A, const float4* Dp, float4* warm)
{
    const size_t smem = FusedShape<MODE>::smem;
    const int grid = resident_grid<k_fused<MODE>>(128, smem, ((((long long)M + 15) >> 4) + 3) / 4);
    k_fused<MODE><<<grid, 128, smem, st>>>(X, ldx, M, W1, b1, W2, b2, hout, ldh, pq, A, Dp, warm);
}

__device__ __forceinline__ float tofloat(float v) { return v; }
__device__ __forceinline__ float tofloat(bf16 v) { return __bfloat162float(v); }

// Per-block partial weight gradients: block b writes
//   part[b][n*K + k] = sum over its rows of dY[r][n] X[r][k]   (n < nout, k < K)
//   part[b][nout*K + n] = sum over its rows of dY[r][n]
// (grid-stride over tiles of 32 rows; each thread owns up to 32 outputs in
// registers).  k_sum_parts then adds the blocks in a fixed order, so the
// gradients are bitwise reproducible.
template <typename TY, typename TX>
__global__ void __launch_bounds__(256) k_wgrad(const TY* __restrict__ dY, int ldy, int nout, const TX* __restrict__ X,
                                               int ldx, int K, int M, float* __restrict__ part)
{
    constexpr int RT = 32, NT = 256, MAXO = 32;
    __shared__ float sy[RT][2 * H + 1];
    __shared__ float sx[RT][2 * H + 1];
    const int nouts = nout * K;
    float acc[MAXO];
    float bacc = 0.f;
    #pragma unroll
    for (int j = 0; j < MAXO; ++j) acc[j] = 0.f;
    for (int r0 = blockIdx.x * RT; r0 < M; r0 += gridDim.x * RT) {
        __syncthreads();
        for (int i = threadIdx.x; i < RT * nout; i += NT) {
            const int r = i / nout, n = i % nout;
            sy[r][n] = r0 + r < M ? tofloat(dY[(size_t)(r0 + r) * ldy + n]) : 0.f;
        }
        for (int i = threadIdx.x; i < RT * K; i += NT) {
            const int r = i / K, k = i % K;
            sx[r][k] = r0 + r < M ? tofloat(X[(size_t)(r0 + r) * ldx + k]) : 0.f;
        }
        __syncthreads();
        #pragma unroll
        for (int j = 0; j < MAXO; ++j) {
            const int o = threadIdx.x + j * NT;
            if (o < nouts) {
                const int n = o / K, k = o % K;
                float s = 0.f;
                #pragma unroll 8
                for (int r = 0; r < RT; ++r) s += sy[r][n] * sx[r][k];
                acc[j] += s;
            }
        }
        if (threadIdx.x < nout)
            for (int r = 0; r < RT; ++r) bacc += sy[r][threadIdx.x];
    }
    float* row = part + (size_t)blockIdx.x * (nouts + nout);
    #pragma unroll
    for (int j = 0; j < MAXO; ++j) {
        const int o = threadIdx.x + j * NT;
        if (o < nouts) row[o] = acc[j];
    }
    if (threadIdx.x < nout) row[nouts + threadIdx.x] = bacc;
}

// dW[i] = sum_b part[b][i] (i < nw), db[i] = sum_b part[b][nw + i] (i < nb,
// db may be null), blocks added in order b = 0, 1, ...
__global__ void k_sum_parts(const float* __restrict__ part, int nblocks, int nw, int nbias, float* __restrict__ dW,
                            float* __restrict__ db)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int width = nw + nbias;
    if (i >= width || (i >= nw && !db)) return;
    float s = 0.f;
    for (int b = 0; b < nblocks; ++b) s += part[(size_t)b * width + i];
    if (i < nw) dW[i] = s; else db[i - nw] = s;
}

// Messages of layer l:
//   a_i = deg_inv_i * sum_j relu(P_i + Q_j + C e_ij + c), written to cat[:, H:2H].
// Half a warp per node, lane s of a half owning channels 4s..4s+3; each warp
// walks pairs of nodes with a grid stride (msg_grid sizes the grid to the
// resident blocks).  A half reads its node's neighbour indices 16 at a time,
// one per lane, and broadcasts them by shuffles; the Q rows and edge
// features of two edges are loaded before either is summed, so their
// latencies overlap.  Each node sums its edges in list order, one at a time;
// channel pairs go through the two-lane fp32 instructions, which round each
// lane like the scalar add and fused multiply-add.
__global__ void __launch_bounds__(256) k_msg_fwd(int N, const int* __restrict__ ptr, const int* __restrict__ adj,
                                                 const float4* __restrict__ ef, const float* __restrict__ deg_inv,
                                                 const bf16* __restrict__ PQ, const float* __restrict__ C,
                                                 const float* __restrict__ cb, bf16* __restrict__ cat)
{
    const unsigned full = 0xffffffffu;
    const int s = threadIdx.x & 15, ch = 4 * s;
    float4 Cw[4];
    float cv[4];
    #pragma unroll
    for (int k = 0; k < 4; ++k) { Cw[k] = *reinterpret_cast<const float4*>(C + (ch + k) * EF); cv[k] = cb[ch + k]; }
    const int npair = (N + 1) >> 1, stride = gridDim.x * (blockDim.x >> 5);
    // the pair index is the same for the whole warp, so every lane takes
    // part in every shuffle below
    for (int pair = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; pair < npair; pair += stride) {
        const int node = 2 * pair + ((threadIdx.x >> 4) & 1);
        const bool live = node < N;
        int e0 = 0, deg = 0;
        float P[4] = {0.f, 0.f, 0.f, 0.f};
        if (live) {
            e0 = ptr[node];
            deg = ptr[node + 1] - e0;
            const uint2 pr = *reinterpret_cast<const uint2*>(PQ + (size_t)node * 2 * H + ch);
            const float2 p01 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&pr.x));
            const float2 p23 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&pr.y));
            P[0] = p01.x; P[1] = p01.y; P[2] = p23.x; P[3] = p23.y;
        }
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        // steps over the larger degree of the warp's two nodes
        const int dmax = max(deg, __shfl_xor_sync(full, deg, 16));
        for (int base = 0; base < dmax; base += 16) {
            const int n = deg - base;   // edges of this node left (may be <= 0)
            const int jl = s < n ? adj[e0 + base + s] : 0;
            const int m = min(16, dmax - base);
            for (int t0 = 0; t0 < m; t0 += 2) {
                int j[2];
                uint2 qr[2];
                float4 f[2];
                #pragma unroll
                for (int u = 0; u < 2; ++u) j[u] = __shfl_sync(full, jl, (t0 + u) & 15, 16);
                #pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const bool ok = t0 + u < n;
                    qr[u] = ok ? *reinterpret_cast<const uint2*>(PQ + (size_t)j[u] * 2 * H + H + ch) : make_uint2(0u, 0u);
                    f[u] = ok ? ef[e0 + base + t0 + u] : make_float4(0.f, 0.f, 0.f, 0.f);
                }
                #pragma unroll
                for (int u = 0; u < 2; ++u) {
                    if (t0 + u < n) {
                        const float2 q01 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&qr[u].x));
                        const float2 q23 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&qr[u].y));
                        float2 z01 = __fadd2_rn(make_float2(P[0], P[1]), q01);
                        float2 z23 = __fadd2_rn(make_float2(P[2], P[3]), q23);
                        z01 = __ffma2_rn(make_float2(Cw[0].x, Cw[1].x), make_float2(f[u].x, f[u].x), z01);
                        z23 = __ffma2_rn(make_float2(Cw[2].x, Cw[3].x), make_float2(f[u].x, f[u].x), z23);
                        z01 = __ffma2_rn(make_float2(Cw[0].y, Cw[1].y), make_float2(f[u].y, f[u].y), z01);
                        z23 = __ffma2_rn(make_float2(Cw[2].y, Cw[3].y), make_float2(f[u].y, f[u].y), z23);
                        z01 = __ffma2_rn(make_float2(Cw[0].z, Cw[1].z), make_float2(f[u].z, f[u].z), z01);
                        z23 = __ffma2_rn(make_float2(Cw[2].z, Cw[3].z), make_float2(f[u].z, f[u].z), z23);
                        z01 = __ffma2_rn(make_float2(Cw[0].w, Cw[1].w), make_float2(f[u].w, f[u].w), z01);
                        z23 = __ffma2_rn(make_float2(Cw[2].w, Cw[3].w), make_float2(f[u].w, f[u].w), z23);
                        z01 = __fadd2_rn(z01, make_float2(cv[0], cv[1]));
                        z23 = __fadd2_rn(z23, make_float2(cv[2], cv[3]));
                        const float2 a01 =
                            __fadd2_rn(make_float2(acc[0], acc[1]), make_float2(fmaxf(z01.x, 0.f), fmaxf(z01.y, 0.f)));
                        const float2 a23 =
                            __fadd2_rn(make_float2(acc[2], acc[3]), make_float2(fmaxf(z23.x, 0.f), fmaxf(z23.y, 0.f)));
                        acc[0] = a01.x; acc[1] = a01.y; acc[2] = a23.x; acc[3] = a23.y;
                    }
                }
            }
        }
        if (live) {
            const float di = deg_inv[node];
            __nv_bfloat162 o[2] = {__floats2bfloat162_rn(acc[0] * di, acc[1] * di),
                                   __floats2bfloat162_rn(acc[2] * di, acc[3] * di)};
            *reinterpret_cast<uint2*>(cat + (size_t)node * 2 * H + H + ch) = *reinterpret_cast<const uint2*>(o);
        }
    }
}

// Grid of k_msg_fwd for N nodes: one warp per pair of nodes, at most the
// blocks that are resident at once on this device.
inline int msg_grid(int N) { return resident_grid<k_msg_fwd>(256, 0, ((((long long)N + 1) >> 1) + 7) / 8); }

// Backward of the messages: dP_i = sum_j g_ij, dQ_j = sum_i g_ij with
// g_ij = [z_ij > 0] da_i / deg_i (da = dcat[:, H:2H]); dC, dc reduced per
// block into `part`.  Each warp handles node n as receiver (dP) and as sender (dQ, via
// the reverse edge's features).
__global__ void __launch_bounds__(256) k_msg_bwd(int N, const int* __restrict__ ptr, const int* __restrict__ adj,
                                                 const int* __restrict__ rev, const float4* __restrict__ ef,
                                                 const float* __restrict__ deg_inv, const bf16* __restrict__ PQ,
                                                 const float* __restrict__ C, const float* __restrict__ cb,
                                                 const float* __restrict__ dcat, float* __restrict__ dpq,
                                                 float* __restrict__ part)
{
    __shared__ float red[8][H * (EF + 1)];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, ch = 2 * lane;
    const float4 C0 = *reinterpret_cast<const float4*>(C + ch * EF), C1 = *reinterpret_cast<const float4*>(C + (ch + 1) * EF);
    const float c0 = cb[ch], c1 = cb[ch + 1];
    float gC[2][EF] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
    float gc0 = 0.f, gc1 = 0.f;
    for (int node = blockIdx.x * 8 + warp; node < N; node += gridDim.x * 8) {
        const float2 Pn = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(PQ + (size_t)node * 2 * H + ch));
        const float2 Qn = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(PQ + (size_t)node * 2 * H + H + ch));
        const float2 dan = *reinterpret_cast<const float2*>(dcat + (size_t)node * 2 * H + H + ch);
        const float din = deg_inv[node];
        float dP0 = 0.f, dP1 = 0.f, dQ0 = 0.f, dQ1 = 0.f;
        for (int e = ptr[node]; e < ptr[node + 1]; ++e) {
            const int j = adj[e];
            // node as receiver of j
            {
                const float4 f = ef[e];
                const float2 Q = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(PQ + (size_t)j * 2 * H + H + ch));
                const float z0 = Pn.x + Q.x + C0.x * f.x + C0.y * f.y + C0.z * f.z + C0.w * f.w + c0;
                const float z1 = Pn.y + Q.y + C1.x * f.x + C1.y * f.y + C1.z * f.z + C1.w * f.w + c1;
                const float g0 = z0 > 0.f ? dan.x * din : 0.f, g1 = z1 > 0.f ? dan.y * din : 0.f;
                dP0 += g0; dP1 += g1;
                gC[0][0] += g0 * f.x; gC[0][1] += g0 * f.y; gC[0][2] += g0 * f.z; gC[0][3] += g0 * f.w;
                gC[1][0] += g1 * f.x; gC[1][1] += g1 * f.y; gC[1][2] += g1 * f.z; gC[1][3] += g1 * f.w;
                gc0 += g0; gc1 += g1;
            }
            // node as sender to j: edge (j <- node) is rev[e] in j's list
            {
                const float4 f = ef[rev[e]];
                const float2 P = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(PQ + (size_t)j * 2 * H + ch));
                const float2 da = *reinterpret_cast<const float2*>(dcat + (size_t)j * 2 * H + H + ch);
                const float dj = deg_inv[j];
                const float z0 = P.x + Qn.x + C0.x * f.x + C0.y * f.y + C0.z * f.z + C0.w * f.w + c0;
                const float z1 = P.y + Qn.y + C1.x * f.x + C1.y * f.y + C1.z * f.z + C1.w * f.w + c1;
                dQ0 += z0 > 0.f ? da.x * dj : 0.f;
                dQ1 += z1 > 0.f ? da.y * dj : 0.f;
            }
        }
        *reinterpret_cast<float2*>(dpq + (size_t)node * 2 * H + ch) = make_float2(dP0, dP1);
        *reinterpret_cast<float2*>(dpq + (size_t)node * 2 * H + H + ch) = make_float2(dQ0, dQ1);
    }
    for (int f = 0; f < EF; ++f) { red[warp][ch * EF + f] = gC[0][f]; red[warp][(ch + 1) * EF + f] = gC[1][f]; }
    red[warp][H * EF + ch] = gc0;
    red[warp][H * EF + ch + 1] = gc1;
    __syncthreads();
    // the block's partial dC (H x EF) then dc (H), summed over blocks in
    // order by k_sum_parts
    for (int i = threadIdx.x; i < H * (EF + 1); i += 256) {
        float s = 0.f;
        for (int w = 0; w < 8; ++w) s += red[w][i];
        part[(size_t)blockIdx.x * H * (EF + 1) + i] = s;
    }
}

// Error d_i = (out_i[0:3] - target_i) w_i over free vertices (w in {0, 1}):
//   loss = inv_cnt [ sum_i |d_i|^2 + lam/2 sum_(i,j) k_ij w_i w_j |d_i - d_j|^2 ]
// over the directed edges (i, j) of the symmetric adjacency, with edge
// weights k_ij (ew; null: 1).  The second term weighs the error's
// differences between neighbours (its high-frequency part); with k_ij from
// the PD system's diagonal it is the energy norm e^T (M + K) e / m of the
// error, K approximated by a graph Laplacian with K's own diagonal.
// dout_i = inv_cnt [2 d_i + 2 lam sum_j k_ij w_j (d_i - d_j)] w_i, one thread
// per vertex, no atomics.
__global__ void k_loss(int N, const float* __restrict__ out, const float* __restrict__ target,
                       const float* __restrict__ freew, const int* __restrict__ ptr, const int* __restrict__ adj,
                       const float* __restrict__ ew, float lam, float inv_cnt, float* __restrict__ dout,
                       double* __restrict__ loss)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float s = 0.f;
    if (i < N) {
        const float w = freew[i];
        float d[NO], gsum[NO];
        #pragma unroll
        for (int c = 0; c < NO; ++c) {
            d[c] = (out[(size_t)i * 16 + c] - target[(size_t)i * 3 + c]) * w;
            s += d[c] * d[c];
            gsum[c] = d[c];
        }
        if (lam != 0.f && w > 0.f) {
            for (int q = ptr[i]; q < ptr[i + 1]; ++q) {
                const int j = adj[q];
                const float wj = freew[j] * (ew ? ew[q] : 1.f);
                if (wj == 0.f) continue;
                float e2 = 0.f;
                #pragma unroll
                for (int c = 0; c < NO; ++c) {
                    const float e = d[c] - (out[(size_t)j * 16 + c] - target[(size_t)j * 3 + c]) * freew[j];
                    e2 += e * e;
                    gsum[c] += lam * wj * e;
                }
                s += 0.5f * lam * wj * e2;
            }
        }
        for (int c = 0; c < 16; ++c) dout[(size_t)i * 16 + c] = c < NO ? 2.f * gsum[c] * w * inv_cnt : 0.f;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0 && s != 0.f) atomicAdd(loss, (double)s * inv_cnt);
}

// dst = src * mask(ref > 0) (ReLU backward; ref is the bf16 ReLU output)
__global__ void k_relu_bwd(int N, int cols, const float* __restrict__ src, int lds, const bf16* __restrict__ ref,
                           int ldr, float* __restrict__ dst, int ldd)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N * cols) return;
    const int r = i / cols, c = i % cols;
    dst[(size_t)r * ldd + c] = __bfloat162float(ref[(size_t)r * ldr + c]) > 0.f ? src[(size_t)r * lds + c] : 0.f;
}

// dst[:, 0:cols] += src[:, 0:cols]
__global__ void k_add(int N, int cols, const float* __restrict__ src, int lds, float* __restrict__ dst, int ldd)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N * cols) return;
    const int r = i / cols, c = i % cols;
    dst[(size_t)r * ldd + c] += src[(size_t)r * lds + c];
}

__global__ void k_adam(int n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr, float b1, float b2, float eps, float bc1, float bc2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

// bf16 copy of a [rows][cols] fp32 tensor into dst[rows_pad][ld] (and its
// transpose into dstT[cols][ldT]); padding rows/cols are left as zero.
__global__ void k_to_bf16(const float* __restrict__ src, int rows, int cols, bf16* __restrict__ dst, int ld,
                          bf16* __restrict__ dstT, int ldT)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * cols) return;
    const int r = i / cols, c = i % cols;
    const bf16 b = __float2bfloat16_rn(src[i]);
    if (dst) dst[(size_t)r * ld + c] = b;
    if (dstT) dstT[(size_t)c * ldT + r] = b;
}

// ---- solver-side feature kernels -----------------------------------------
// Node features: (y - x)/s, h v / s, pinned, scaled log mass / log stretch k /
// log bend k, then the previous frame's offset d_prev / s and its validity
// (Dp.w: 1 when the vertex's state entering the frame is the one the solver
// left after its previous frame, else 0 and d_prev = 0).
__global__ void k_node_feat(int N, const float4* __restrict__ X, const float4* __restrict__ V,
                            const float4* __restrict__ Y, const float4* __restrict__ aux,
                            const float4* __restrict__ stat, const int* __restrict__ vcloth,
                            const ClothInfo* __restrict__ cinfo, const float4* __restrict__ Dp,
                            bf16* __restrict__ xin)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const float4 x = X[i], v = V[i], y = Y[i], s = stat[i];
    const float4 dp = Dp ? Dp[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float ok = dp.w > 0.f ? 1.f : 0.f;
    const float h = cinfo[vcloth[i]].h, is = 1.f / kOffsetScale;
    float f[NFP];
    f[0] = (y.x - x.x) * is; f[1] = (y.y - x.y) * is; f[2] = (y.z - x.z) * is;
    f[3] = h * v.x * is; f[4] = h * v.y * is; f[5] = h * v.z * is;
    f[6] = aux[i].w < 0.f ? 1.f : 0.f;
    f[7] = s.x; f[8] = s.y; f[9] = s.z;
    f[10] = ok * dp.x * is; f[11] = ok * dp.y * is; f[12] = ok * dp.z * is;
    f[13] = ok;
    for (int k = NF; k < NFP; ++k) f[k] = 0.f;
    for (int k = 0; k < NFP; k += 2)
        *reinterpret_cast<__nv_bfloat162*>(xin + (size_t)i * NFP + k) = __floats2bfloat162_rn(f[k], f[k + 1]);
}

// edge features of (i <- j): log(rest / 1 cm), (y_j - y_i) / rest
__global__ void k_edge_feat(int N, const int* __restrict__ ptr, const int* __restrict__ adj,
                            const float* __restrict__ rest, const float4* __restrict__ Y, float4* __restrict__ ef)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const float4 yi = Y[i];
    for (int e = ptr[i]; e < ptr[i + 1]; ++e) {
        const float4 yj = Y[adj[e]];
        const float r = rest[e], ir = 1.f / r;
        ef[e] = make_float4(logf(r / kLenScale), (yj.x - yi.x) * ir, (yj.y - yi.y) * ir, (yj.z - yi.z) * ir);
    }
}

// Target of the network: (x* - y - d_prev)/s, i.e. the change of the
// converged offset since the previous frame where d_prev is valid (the
// prediction adds d_prev back, a skip connection in fp32), and the free weight.
__global__ void k_target(int N, const float4* __restrict__ Xs, const float4* __restrict__ Y,
                         const float4* __restrict__ aux, const float4* __restrict__ Dp, float* __restrict__ target,
                         float* __restrict__ freew)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const float4 x = Xs[i], y = Y[i];
    const float4 dp = Dp ? Dp[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float ok = dp.w > 0.f ? 1.f : 0.f;
    const float is = 1.f / kOffsetScale;
    target[3 * i] = (x.x - y.x - ok * dp.x) * is;
    target[3 * i + 1] = (x.y - y.y - ok * dp.y) * is;
    target[3 * i + 2] = (x.z - y.z - ok * dp.z) * is;
    freew[i] = aux[i].w < 0.f ? 0.f : 1.f;
}

}  // namespace gnn
}  // namespace pdg
