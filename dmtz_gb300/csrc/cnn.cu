// cnn.cu — the learned proposal: a 4-layer 3x3x3 convolutional network with
// BF16 weights/activations and FP32 accumulation on the tensor cores, its
// backward pass, and the loss / optimiser kernels.  No counterpart in the
// reference; it only produces a starting point for the exact correction loop.
//
// Layout: activations channels-last bf16, [vertex][channel], vertex =
// x + W*(y + H*z).  Layers (in -> out channels): 16 -> 32 -> 32 -> 32 -> 16,
// ReLU after the first three; only output channel 0 is used (the other 15
// have zero weights and zero gradients, so they stay zero).  Parameters (f32
// master copy), per layer: weights [27 taps][out][in], then bias [out];
// tap = (dz+1)*9 + (dy+1)*3 + (dx+1).
//
// Kernels (all persistent: one or two blocks per SM loop over tiles):
//   k_conv_tc  the convolutions (forward and data gradient) on tcgen05: a
//            tile of 128 vertices per MMA chain, accumulator in tensor
//            memory (the default path; see its comment).
//   k_conv   the same convolution on mma.sync.m16n8k16 (bf16 in, f32
//            accumulate).  A block keeps all 27 x out x in weights in shared
//            memory and streams 8x8x4-vertex tiles (+1 halo) through a
//            cp.async double buffer; operands reach registers by ldmatrix.
//            The data gradient is the same kernel with transposed weights,
//            mirrored taps and a ReLU-derivative epilogue.
//   k_wgrad  weight + bias gradient: per tile, all 27 taps x out x in
//            products reduced over the tile's 256 vertices on the same MMA
//            (operands by ldmatrix.trans from the channels-last tiles);
//            per-block partial sums, then a fixed-order reduction
//            (deterministic).
//   k_loss, k_loss_final, k_reduce, k_adam, k_pack: loss, gradient scaling,
//            Adam, bf16 weight refresh.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "cnn.cuh"

typedef __nv_bfloat16 bf16;
typedef long long i64;

namespace {

constexpr int TX = 8, TY = 8, TZ = 4, TV = TX * TY * TZ;  // output tile (256 vertices)
constexpr int HX = TX + 2, HY = TY + 2, HZ = TZ + 2, HALO = HX * HY * HZ;
constexpr int NLAYER = 4;
constexpr int LCIN[NLAYER] = {16, 32, 32, 32};
constexpr int LCOUT[NLAYER] = {32, 32, 32, 16};

constexpr i64 layer_params(int l) { return 27LL * LCOUT[l] * LCIN[l] + LCOUT[l]; }
constexpr i64 layer_offset(int l) { return l == 0 ? 0 : layer_offset(l - 1) + layer_params(l - 1); }
constexpr i64 kParams = layer_offset(NLAYER);

// ------------------------------------------------------------------ PTX helpers
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
// 16-byte async copy global -> shared; src_bytes = 0 writes zeros (the source
// address is not read then, but is kept valid anyway)
__device__ __forceinline__ void cp16(void *dst, const void *src, int src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_addr(dst)), "l"(src), "r"(src_bytes));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}
__device__ __forceinline__ void ldm4(uint32_t r[4], const void *p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_addr(p)));
}
__device__ __forceinline__ void ldm4t(uint32_t r[4], const void *p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_addr(p)));
}
__device__ __forceinline__ void mma16816(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

struct Dims {
    int W, H, D, ntx, nty, ntz;
    i64 ntiles;
};
inline Dims make_dims(int W, int H, int D) {
    Dims d{W, H, D, (W + TX - 1) / TX, (H + TY - 1) / TY, (D + TZ - 1) / TZ, 0};
    d.ntiles = (i64)d.ntx * d.nty * d.ntz;
    return d;
}

// Box of EX x EY x EZ vertices starting at (x0, y0, z0) (may stick out of the
// grid: zeros there) of a channels-last tensor with C channels, into shared
// rows of CP = C + 8 bf16 (the 16-byte pad makes ldmatrix conflict-free).
template <int C, int EX, int EY, int EZ>
__device__ __forceinline__ void load_box(bf16 *dst, const bf16 *__restrict__ src, const Dims &d, int x0, int y0,
                                         int z0) {
    constexpr int CP = C + 8, PIECES = C / 8;
    for (int i = threadIdx.x; i < EX * EY * EZ * PIECES; i += blockDim.x) {
        const int row = i / PIECES, piece = i - row * PIECES;
        const int hx = row % EX, hy = (row / EX) % EY, hz = row / (EX * EY);
        const int gx = x0 + hx, gy = y0 + hy, gz = z0 + hz;
        const bool in = gx >= 0 && gx < d.W && gy >= 0 && gy < d.H && gz >= 0 && gz < d.D;
        const bf16 *s = in ? src + ((i64)gx + (i64)gy * d.W + (i64)gz * d.W * d.H) * C + piece * 8 : src;
        cp16(dst + row * CP + piece * 8, s, in ? 16 : 0);
    }
}

__device__ __forceinline__ void tile_origin(const Dims &d, i64 tile, int &x0, int &y0, int &z0) {
    x0 = (int)(tile % d.ntx) * TX;
    y0 = (int)((tile / d.ntx) % d.nty) * TY;
    z0 = (int)(tile / ((i64)d.ntx * d.nty)) * TZ;
}

}  // namespace

namespace {

// ---------------------------------------------------------------- convolution
// out[v][n] = sum_tap sum_c W[tap][n][c] * in[v + off(tap)][c]   (FLIP: v - off)
// MODE 0: + bias, ReLU, bf16 out.  MODE 1: + bias, channel 0 as f32 (the
// proposal).  MODE 2 (data gradient): no bias; zero where aux, the stored
// activation that fed the layer, is not positive (ReLU derivative).
// 8 warps; warp w owns tile vertices 32w..32w+31 (two m16 tiles), all COUT.
template <int CIN, int COUT, int MODE, bool FLIP>
__global__ void __launch_bounds__(256, 1) k_conv(Dims d, const bf16 *__restrict__ in, const bf16 *__restrict__ wt,
                                              const float *__restrict__ bias, void *out,
                                              const bf16 *__restrict__ aux) {
    constexpr int CP = CIN + 8, NT = COUT / 8, KC = CIN / 16;
    static_assert(NT % 2 == 0 && CIN % 16 == 0, "tile shapes");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    bf16 *ws = reinterpret_cast<bf16 *>(smem_raw);  // [27*COUT][CP]
    bf16 *xs0 = ws + 27 * COUT * CP;                 // 2 x [HALO][CP]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
    for (int i = tid; i < 27 * COUT * (CIN / 8); i += blockDim.x) {
        const int row = i / (CIN / 8), piece = i - row * (CIN / 8);
        cp16(ws + row * CP + piece * 8, wt + (i64)row * CIN + piece * 8, 16);
    }
    // ldmatrix roles.  A (vertices x channels): lane supplies row
    // (lane&7) + 8*((lane>>3)&1) of the m-tile, channel half 8*(lane>>4).
    // B (weights, rows = output channel): n = 8*(lane>>4) + (lane&7) within a
    // pair of n-tiles, channel half 8*((lane>>3)&1).
    int hbase[2];
#pragma unroll
    for (int m = 0; m < 2; m++) {
        const int li = warp * 32 + m * 16 + (lane & 7) + 8 * ((lane >> 3) & 1);
        hbase[m] = (((li >> 6) + 1) * HY + ((li >> 3) & 7) + 1) * HX + (li & 7) + 1;
    }
    const int akofs = 8 * (lane >> 4);
    const int bn = 8 * (lane >> 4) + (lane & 7), bkofs = 8 * ((lane >> 3) & 1);

    i64 tile = blockIdx.x;
    int buf = 0;
    if (tile < d.ntiles) {
        int x0, y0, z0;
        tile_origin(d, tile, x0, y0, z0);
        load_box<CIN, HX, HY, HZ>(xs0, in, d, x0 - 1, y0 - 1, z0 - 1);
    }
    cp_commit();
    for (; tile < d.ntiles; tile += gridDim.x, buf ^= 1) {
        const i64 next = tile + gridDim.x;
        if (next < d.ntiles) {
            int x0, y0, z0;
            tile_origin(d, next, x0, y0, z0);
            load_box<CIN, HX, HY, HZ>(xs0 + (buf ^ 1) * HALO * CP, in, d, x0 - 1, y0 - 1, z0 - 1);
        }
        cp_commit();
        cp_wait<1>();
        __syncthreads();
        const bf16 *xs = xs0 + buf * HALO * CP;
        float acc[2][NT][4];
#pragma unroll
        for (int m = 0; m < 2; m++)
#pragma unroll
            for (int n = 0; n < NT; n++)
#pragma unroll
                for (int k = 0; k < 4; k++) acc[m][n][k] = 0.f;
#pragma unroll 1
        for (int tap = 0; tap < 27; tap++) {
            const int dx = tap % 3 - 1, dy = (tap / 3) % 3 - 1, dzz = tap / 9 - 1;
            const int toff = FLIP ? -((dzz * HY + dy) * HX + dx) : (dzz * HY + dy) * HX + dx;
            const bf16 *wtap = ws + tap * COUT * CP;
#pragma unroll
            for (int kc = 0; kc < KC; kc++) {
                uint32_t a0[4], a1[4];
                ldm4(a0, xs + (hbase[0] + toff) * CP + kc * 16 + akofs);
                ldm4(a1, xs + (hbase[1] + toff) * CP + kc * 16 + akofs);
#pragma unroll
                for (int j = 0; j < NT; j += 2) {
                    uint32_t b[4];
                    ldm4(b, wtap + (j * 8 + bn) * CP + kc * 16 + bkofs);
                    mma16816(acc[0][j], a0, b[0], b[1]);
                    mma16816(acc[1][j], a1, b[0], b[1]);
                    mma16816(acc[0][j + 1], a0, b[2], b[3]);
                    mma16816(acc[1][j + 1], a1, b[2], b[3]);
                }
            }
        }
        // accumulator (m, n, k): vertex row g + 8*(k>>1), channel n*8 + 2t + (k&1)
        int x0, y0, z0;
        tile_origin(d, tile, x0, y0, z0);
#pragma unroll
        for (int m = 0; m < 2; m++)
#pragma unroll
            for (int r = 0; r < 2; r++) {
                const int li = warp * 32 + m * 16 + g + 8 * r;
                const int gx = x0 + (li & 7), gy = y0 + ((li >> 3) & 7), gz = z0 + (li >> 6);
                if (gx >= d.W || gy >= d.H || gz >= d.D) continue;
                const i64 v = gx + (i64)gy * d.W + (i64)gz * d.W * d.H;
                if constexpr (MODE == 1) {
                    if (t == 0) reinterpret_cast<float *>(out)[v] = acc[m][0][2 * r] + bias[0];
                } else {
#pragma unroll
                for (int n = 0; n < NT; n++) {
                    const int ch = n * 8 + 2 * t;
                    float v0 = acc[m][n][2 * r], v1 = acc[m][n][2 * r + 1];
                    if constexpr (MODE == 0) {
                        v0 = fmaxf(v0 + bias[ch], 0.f);
                        v1 = fmaxf(v1 + bias[ch + 1], 0.f);
                    } else {
                        const __nv_bfloat162 a2 = *reinterpret_cast<const __nv_bfloat162 *>(aux + v * COUT + ch);
                        if (!(__bfloat162float(a2.x) > 0.f)) v0 = 0.f;
                        if (!(__bfloat162float(a2.y) > 0.f)) v1 = 0.f;
                    }
                    *reinterpret_cast<__nv_bfloat162 *>(reinterpret_cast<bf16 *>(out) + v * COUT + ch) =
                        __floats2bfloat162_rn(v0, v1);
                }
                }
            }
        __syncthreads();  // buffer `buf` is refilled two iterations on
    }
    cp_wait<0>();
}

// ------------------------------------------------- convolution on tcgen05
// The same convolution (same modes, FLIP, epilogues) on the 5th-generation
// tensor cores: tcgen05.mma with the accumulator in tensor memory.
//
// GEMM per z-slice of a tile: D[128 vertices][COUT] = sum over 27 taps of
// A_tap[128][CIN] x W_tap[CIN][COUT], K = 16 per instruction.  A tile is
// 8 x 16 x 4 vertices (x, y, z): four slices whose 128 rows are 16 lines of
// 8 x-neighbours.  Its halo box (10 x 18 x 6 vertices) sits in shared memory
// as CIN/8 planes, one per 16-byte group of 8 channels, each plane
// vertex-major (16 bytes per vertex).  In that layout the 8 rows of one
// x-line and one channel group are 128 contiguous bytes: one "core matrix" of
// the no-swizzle K-major operand layout.  A tap's A operand is the box
// shifted by the tap's offset: its descriptor starts at the shifted vertex,
// steps 10 x 16 bytes from one line to the next (stride byte offset) and one
// plane from one channel group to the next (leading byte offset).  Weights
// are stored per tap as [group][out channel][8 channels], the same layout for
// B.  The boxes arrive by TMA; the roles that issue the MMAs and copies and
// run the epilogue are described at k_conv_tc.
constexpr int QX = 8, QY = 16, QZ = 4;  // tile: QZ slices of 128 vertices (one MMA chain each)
constexpr int GX = QX + 2, GY = QY + 2, GZ = QZ + 2, GVOX = GX * GY * GZ;  // halo box
inline Dims make_tc_dims(int W, int H, int D) {
    Dims d{W, H, D, (W + QX - 1) / QX, (H + QY - 1) / QY, (D + QZ - 1) / QZ, 0};
    d.ntiles = (i64)d.ntx * d.nty * d.ntz;
    return d;
}
__device__ __forceinline__ void tc_tile_origin(const Dims &d, i64 tile, int &x0, int &y0, int &z0) {
    x0 = (int)(tile % d.ntx) * QX;
    y0 = (int)((tile / d.ntx) % d.nty) * QY;
    z0 = (int)(tile / ((i64)d.ntx * d.nty)) * QZ;
}
// shared-memory matrix descriptor: no swizzle, start / leading / stride byte
// offsets in 16-byte units, descriptor version 1 (bit 46)
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// instruction descriptor of kind::f16: f32 accumulator, bf16 A and B, both
// K-major, N = COUT, M = 128
template <int COUT>
__device__ __forceinline__ uint32_t tc_idesc() {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(COUT >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}
__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.u32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int limit) {
    uint32_t done = 0;
    for (int it = 0; it < limit && !done; it++)
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity));
    return done != 0;
}
// this warp's 32 accumulator rows, columns 0..N-1 (N = 16 or 32), into r;
// the registers are valid after tmem_wait()
template <int N>
__device__ __forceinline__ void tmem_ld(uint32_t taddr, uint32_t (&r)[N]) {
    if constexpr (N == 32) {
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
              "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
              "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
              "=r"(r[30]), "=r"(r[31])
            : "r"(taddr));
    } else {
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
            "[%16];\n"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
            : "r"(taddr));
    }
}
__device__ __forceinline__ void tmem_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }
// The halo box arrives by TMA: the activations are a 4-d tensor (channel,
// x, y, z) with a box of (8 channels, GX, GY, GZ), so one bulk copy per
// 8-channel group writes exactly one plane (vertex-major, 16 bytes per
// vertex), zeros outside the grid.  The box starts at channel 8c (16-byte
// aligned, as a tiled copy's innermost coordinate must be) and at the halo's
// corner (x0-1, y0-1, z0-1), which may be -1.  Planes are padded to a
// multiple of 128 bytes (bulk-copy destinations).
constexpr uint32_t TC_PLANE = ((GVOX * 16 + 127) / 128) * 128;
template <int CIN>
__device__ __forceinline__ void tc_issue_box(const CUtensorMap *tm, uint32_t dst, uint32_t bar, int x0, int y0,
                                             int z0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar),
                 "r"((uint32_t)(CIN / 8 * GVOX * 16)));
#pragma unroll
    for (int c = 0; c < CIN / 8; c++)
        asm volatile(
            "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
            "%5}], [%6];\n" ::"r"(dst + c * TC_PLANE),
            "l"(reinterpret_cast<uint64_t>(tm)), "r"(c * 8), "r"(x0 - 1), "r"(y0 - 1), "r"(z0 - 1), "r"(bar)
            : "memory");
}

template <int CIN, int COUT>
constexpr size_t tc_smem() {
    return 128 + (size_t)27 * (CIN / 8) * COUT * 16 + 2 * (size_t)(CIN / 8) * TC_PLANE;
}

// Roles (192 threads): warp 0 lane 0 issues the MMAs, warp 1 lane 0 issues
// the TMA box copies, warps 2..5 run the epilogue (warp w reads accumulator
// lanes 32 (w mod 4) .. 32 (w mod 4) + 31, the quarter tensor memory lets it
// access).  Two box buffers and two accumulator sets (2 x QZ x 32 columns)
// let tile i's MMAs run while tile i-1's epilogue drains its accumulator and
// tile i+1's box arrives.  Barriers, per buffer b:
//   full[b]  the box of the tile using b has landed (TMA complete_tx)
//   mma[b]   that tile's MMAs are done (tcgen05.commit): its accumulator may
//            be read and its box buffer refilled
//   free[b]  the epilogue has read that accumulator (one arrival per
//            epilogue warp)
// Tile i uses b = i mod 2 and completes phase i / 2 of each barrier; every
// wait is bounded, and a role that gives up reports in *err and leaves its
// loop (the others then time out on the phases it no longer completes).
constexpr int kConvThreads = 192;
constexpr int kConvWaitPolls = 1 << 24;
template <int CIN, int COUT, int MODE, bool FLIP>
__global__ void __launch_bounds__(kConvThreads, 1) k_conv_tc(const __grid_constant__ CUtensorMap tmap, Dims d,
                                                           const bf16 *__restrict__ wt, const float *__restrict__ bias,
                                                           void *out, const bf16 *__restrict__ aux, int *err) {
    constexpr int KCH = CIN / 8;
    constexpr uint32_t PLANE = TC_PLANE, WTAP = KCH * COUT * 16, WBYTES = 27 * WTAP, XBYTES = KCH * PLANE;
    constexpr uint32_t ACC_COLS = QZ * 32;  // one accumulator set
    static_assert(CIN % 16 == 0 && (COUT == 16 || COUT == 32), "tile shapes");
    static_assert(WTAP % 128 == 0, "planes stay 128-byte aligned");
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ uint32_t tmem_slot;
    __shared__ __align__(8) uint64_t bar_full[2], bar_mma[2], bar_free[2];
    unsigned char *ws = smem_raw + ((128 - (smem_addr(smem_raw) & 127)) & 127);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int i = tid; i < 27 * COUT * KCH; i += blockDim.x) {
        const int tap = i / (COUT * KCH), rem = i - tap * (COUT * KCH), n = rem / KCH, c = rem - n * KCH;
        cp16(ws + tap * WTAP + c * COUT * 16 + n * 16, wt + ((i64)tap * COUT + n) * CIN + c * 8, 16);
    }
    cp_commit();
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         smem_addr(&tmem_slot)),
                     "n"(2 * ACC_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    // barrier addresses by buffer (selected, not indexed: no local-memory array)
    const uint32_t full0 = smem_addr(&bar_full[0]), full1 = smem_addr(&bar_full[1]);
    const uint32_t mma0 = smem_addr(&bar_mma[0]), mma1 = smem_addr(&bar_mma[1]);
    const uint32_t fre0 = smem_addr(&bar_free[0]), fre1 = smem_addr(&bar_free[1]);
    auto full = [&](int b) { return b ? full1 : full0; };
    auto mma = [&](int b) { return b ? mma1 : mma0; };
    auto fre = [&](int b) { return b ? fre1 : fre0; };
    const uint32_t wbase = smem_addr(ws), xbase0 = wbase + WBYTES;
    if (tid == 0) {
#pragma unroll
        for (int b = 0; b < 2; b++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(full(b)));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mma(b)));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;\n" ::"r"(fre(b)));
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n");
    }
    cp_wait<0>();
    asm volatile("fence.proxy.async.shared::cta;\n");  // the weights, for the tensor core
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    const uint32_t tmem = tmem_slot;
    const i64 first = blockIdx.x, stride = gridDim.x;
    const int ntile = first < d.ntiles ? (int)((d.ntiles - 1 - first) / stride + 1) : 0;
    bool failed = false;

    if (warp == 0) {
        if (lane == 0) {  // MMA issuer
            const uint32_t idesc = tc_idesc<COUT>();
            const uint64_t b0 = smem_desc(wbase, COUT * 16, 128);
            int committed = 0;
            for (int it = 0; it < ntile; it++) {
                const int b = it & 1;
                if (!mbar_wait(full(b), (uint32_t)(it >> 1) & 1u, kConvWaitPolls) ||
                    (it >= 2 && !mbar_wait(fre(b), (uint32_t)((it >> 1) - 1) & 1u, kConvWaitPolls))) {
                    failed = true;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n");
                // descriptors of every (tap, channel group) differ from the
                // buffer's and the weights' base descriptors only in the
                // start-address field (shared addresses stay below 2^18, so
                // adding the offset in 16-byte units never carries out of it):
                // the unrolled chain adds immediates.  The QZ slices' chains
                // are interleaved so that consecutive MMAs go to different
                // accumulators.
                const uint64_t a0 = smem_desc(xbase0 + b * XBYTES, PLANE, GX * 16);
                const uint32_t acc = tmem + (uint32_t)b * ACC_COLS;
#pragma unroll
                for (int tap = 0; tap < 27; tap++) {
                    // offset + 1 along each axis (FLIP mirrors the tap: -d + 1 = 2 - (d + 1))
                    const int sx = FLIP ? 2 - tap % 3 : tap % 3, sy = FLIP ? 2 - (tap / 3) % 3 : (tap / 3) % 3,
                              sz = FLIP ? 2 - tap / 9 : tap / 9;
                    const uint32_t shift = (uint32_t)((sz * GY + sy) * GX + sx) * 16u;
#pragma unroll
                    for (int kk = 0; kk < KCH / 2; kk++)
#pragma unroll
                        for (int q = 0; q < QZ; q++)
                            tc_mma(acc + (uint32_t)(q * 32), a0 + ((shift + q * GY * GX * 16 + kk * 2 * PLANE) >> 4),
                                   b0 + ((tap * WTAP + kk * 2 * COUT * 16) >> 4), idesc, (tap | kk) != 0);
                }
                asm volatile(
                    "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mma(b)));
                committed = it + 1;
            }
            if (committed > 0)  // every MMA issued is done before the accumulators are released
                mbar_wait(mma((committed - 1) & 1), (uint32_t)((committed - 1) >> 1) & 1u, kConvWaitPolls);
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) {  // box producer
            int issued = 0;
            for (int it = 0; it < ntile; it++) {
                const int b = it & 1;
                // buffer b was last read by tile it-2's MMAs
                if (it >= 2 && !mbar_wait(mma(b), (uint32_t)((it >> 1) - 1) & 1u, kConvWaitPolls)) {
                    failed = true;
                    break;
                }
                int x0, y0, z0;
                tc_tile_origin(d, first + it * stride, x0, y0, z0);
                tc_issue_box<CIN>(&tmap, xbase0 + b * XBYTES, full(b), x0, y0, z0);
                issued = it + 1;
            }
            // the copies still in flight land before the block leaves
            for (int j = issued - 2; j < issued; j++)
                if (j >= 0) mbar_wait(full(j & 1), (uint32_t)(j >> 1) & 1u, kConvWaitPolls);
        }
        __syncwarp();
    } else {  // epilogue: warps 2..5
        const int quarter = warp & 3;
        const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16);
        float bsh[COUT];  // the layer's bias, held in registers (MODE 0 adds all, MODE 1 the first)
#pragma unroll
        for (int c = 0; c < COUT; c++) bsh[c] = MODE == 2 ? 0.f : (MODE == 1 && c > 0 ? 0.f : bias[c]);
        for (int it = 0; it < ntile; it++) {
            const int b = it & 1;
            if (!mbar_wait(mma(b), (uint32_t)(it >> 1) & 1u, kConvWaitPolls)) {
                failed = true;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n");
            // every slice's rows at once, one wait, and the accumulator set is
            // handed back to the MMA issuer before the arithmetic and stores
            uint32_t raw[QZ][COUT];
#pragma unroll
            for (int zq = 0; zq < QZ; zq++) tmem_ld<COUT>(taddr + (uint32_t)b * ACC_COLS + (uint32_t)(zq * 32), raw[zq]);
            tmem_wait();
            asm volatile("tcgen05.fence::before_thread_sync;\n");
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(fre(b)) : "memory");
            int x0, y0, z0;
            tc_tile_origin(d, first + it * stride, x0, y0, z0);
            const int r = quarter * 32 + lane, gx = x0 + (r & 7), gy = y0 + (r >> 3);
#pragma unroll
            for (int zq = 0; zq < QZ; zq++) {  // slice zq of the tile
                const int gz = z0 + zq;
                if (gx < d.W && gy < d.H && gz < d.D) {
                    const i64 v = gx + (i64)gy * d.W + (i64)gz * d.W * d.H;
                    if constexpr (MODE == 1) {
                        reinterpret_cast<float *>(out)[v] = __uint_as_float(raw[zq][0]) + bsh[0];
                    } else {
                        uint4 *o = reinterpret_cast<uint4 *>(reinterpret_cast<bf16 *>(out) + v * COUT);
                        const uint4 *ax = MODE == 2 ? reinterpret_cast<const uint4 *>(aux + v * COUT) : nullptr;
#pragma unroll
                        for (int q = 0; q < COUT / 8; q++) {
                            uint4 mk = make_uint4(0, 0, 0, 0);
                            if constexpr (MODE == 2) mk = ax[q];
                            const bf16 *mb = reinterpret_cast<const bf16 *>(&mk);
                            uint4 pk;
                            __nv_bfloat162 *p2 = reinterpret_cast<__nv_bfloat162 *>(&pk);
#pragma unroll
                            for (int h = 0; h < 4; h++) {
                                const int ch = q * 8 + 2 * h;
                                float v0 = __uint_as_float(raw[zq][ch]), v1 = __uint_as_float(raw[zq][ch + 1]);
                                if constexpr (MODE == 0) {
                                    v0 = fmaxf(v0 + bsh[ch], 0.f);
                                    v1 = fmaxf(v1 + bsh[ch + 1], 0.f);
                                } else {
                                    if (!(__bfloat162float(mb[2 * h]) > 0.f)) v0 = 0.f;
                                    if (!(__bfloat162float(mb[2 * h + 1]) > 0.f)) v1 = 0.f;
                                }
                                p2[h] = __floats2bfloat162_rn(v0, v1);
                            }
                            o[q] = pk;
                        }
                    }
                }
            }
        }
    }
    if (failed) atomicOr(err, 1);
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "n"(2 * ACC_COLS));
}

// ---------------------------------------- convolution on tcgen05, x-taps folded
// The same convolution with wider products.  For each (dy, dz) offset one
// MMA multiplies the rows shifted by (-1, dy, dz) with the three x-taps'
// weight blocks side by side (N = 3 COUT): columns [t COUT, (t+1) COUT) of
// row r hold the contribution of x-tap t (dx = t - 1) to the output t
// vertices before row r's along x, so
//   out[r] = D[r][0, COUT) + D[r+1][COUT, 2 COUT) + D[r+2][2 COUT, 3 COUT),
// summed in the epilogue with two warp shuffles per channel.  A tile's 128
// rows are 8 lines of 16 x-neighbours (two core matrices per line, so the
// 8-row groups are 128 bytes apart throughout), of which the first 14 are
// outputs; tiles step 14 along x and overlap by two rows.  The box needs no
// halo along +x (16 x 10 x (QZ2 + 2) vertices).  9 x CIN/16 x QZ2 MMAs per
// tile of 14 x 8 x QZ2 outputs.  Roles, barriers and bounded waits as in
// k_conv_tc; FLIP mirrors the taps through the weight layout.
constexpr int XF_TX = 14, XF_GX = 16, XF_TY = 8, XF_GY = XF_TY + 2, XF_QZ = 2, XF_GZ = XF_QZ + 2;
constexpr int XF_GVOX = XF_GX * XF_GY * XF_GZ;
constexpr uint32_t XF_PLANE = XF_GVOX * 16;  // a multiple of 128
inline Dims make_xf_dims(int W, int H, int D) {
    Dims d{W, H, D, (W + XF_TX - 1) / XF_TX, (H + XF_TY - 1) / XF_TY, (D + XF_QZ - 1) / XF_QZ, 0};
    d.ntiles = (i64)d.ntx * d.nty * d.ntz;
    return d;
}
// accumulator columns of one slice: 3 COUT rounded up to a power of two
template <int COUT>
__host__ __device__ constexpr uint32_t xf_cols() {
    return COUT == 32 ? 128u : 64u;
}
template <int CIN, int COUT>
constexpr size_t xf_smem() {
    return 128 + (size_t)9 * (CIN / 8) * (3 * COUT) * 16 + 2 * (size_t)(CIN / 8) * XF_PLANE;
}
template <int CIN, int COUT, int MODE, bool FLIP>
__global__ void __launch_bounds__(kConvThreads, 1) k_conv_tcx(const __grid_constant__ CUtensorMap tmap, Dims d,
                                                            const bf16 *__restrict__ wt,
                                                            const float *__restrict__ bias, void *out,
                                                            const bf16 *__restrict__ aux, int *err) {
    constexpr int KCH = CIN / 8, N = 3 * COUT;
    constexpr uint32_t WGRP = N * 16, WBYTES = 9 * KCH * WGRP, XBYTES = KCH * XF_PLANE;
    constexpr uint32_t SCOLS = xf_cols<COUT>(), ACC_COLS = XF_QZ * SCOLS, ALLOC = 2 * ACC_COLS;
    static_assert(CIN % 16 == 0 && (COUT == 16 || COUT == 32), "tile shapes");
    static_assert(WGRP % 128 == 0 && XF_PLANE % 128 == 0, "operand blocks stay 128-byte aligned");
    static_assert(ALLOC == 256 || ALLOC == 512, "tensor-memory allocation is a power of two");
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ uint32_t tmem_slot;
    __shared__ __align__(8) uint64_t bar_full[2], bar_mma[2], bar_free[2];
    unsigned char *ws = smem_raw + ((128 - (smem_addr(smem_raw) & 127)) & 127);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // weights: per (dy, dz) offset u and channel group kc, rows n = t COUT + c
    // hold tap (t - 1, dy, dz) of output channel c (mirrored under FLIP)
    for (int i = tid; i < 9 * KCH * N; i += blockDim.x) {
        const int u = i / (KCH * N), rem = i - u * (KCH * N), kc = rem / N, n = rem - kc * N;
        const int t = n / COUT, c = n - t * COUT;
        const int tap = FLIP ? 26 - (t + 3 * u) : t + 3 * u;
        cp16(ws + (u * KCH + kc) * WGRP + n * 16, wt + ((i64)tap * COUT + c) * CIN + kc * 8, 16);
    }
    cp_commit();
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         smem_addr(&tmem_slot)),
                     "n"(ALLOC));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    const uint32_t full0 = smem_addr(&bar_full[0]), full1 = smem_addr(&bar_full[1]);
    const uint32_t mma0 = smem_addr(&bar_mma[0]), mma1 = smem_addr(&bar_mma[1]);
    const uint32_t fre0 = smem_addr(&bar_free[0]), fre1 = smem_addr(&bar_free[1]);
    auto full = [&](int b) { return b ? full1 : full0; };
    auto mma = [&](int b) { return b ? mma1 : mma0; };
    auto fre = [&](int b) { return b ? fre1 : fre0; };
    const uint32_t wbase = smem_addr(ws), xbase0 = wbase + WBYTES;
    if (tid == 0) {
#pragma unroll
        for (int b = 0; b < 2; b++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(full(b)));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mma(b)));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;\n" ::"r"(fre(b)));
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n");
    }
    cp_wait<0>();
    asm volatile("fence.proxy.async.shared::cta;\n");
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    const uint32_t tmem = tmem_slot;
    const i64 first = blockIdx.x, stride = gridDim.x;
    const int ntile = first < d.ntiles ? (int)((d.ntiles - 1 - first) / stride + 1) : 0;
    auto origin = [&](i64 tile, int &x0, int &y0, int &z0) {
        x0 = (int)(tile % d.ntx) * XF_TX;
        y0 = (int)((tile / d.ntx) % d.nty) * XF_TY;
        z0 = (int)(tile / ((i64)d.ntx * d.nty)) * XF_QZ;
    };
    bool failed = false;

    if (warp == 0) {
        if (lane == 0) {  // MMA issuer
            const uint32_t idesc =
                (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
            const uint64_t b0 = smem_desc(wbase, WGRP, 128);
            int committed = 0;
            for (int it = 0; it < ntile; it++) {
                const int b = it & 1;
                if (!mbar_wait(full(b), (uint32_t)(it >> 1) & 1u, kConvWaitPolls) ||
                    (it >= 2 && !mbar_wait(fre(b), (uint32_t)((it >> 1) - 1) & 1u, kConvWaitPolls))) {
                    failed = true;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n");
                const uint64_t a0 = smem_desc(xbase0 + b * XBYTES, XF_PLANE, 128);
                const uint32_t acc = tmem + (uint32_t)b * ACC_COLS;
#pragma unroll
                for (int u = 0; u < 9; u++) {
                    const int sy = u % 3, sz = u / 3;  // dy + 1, dz + 1
#pragma unroll
                    for (int kk = 0; kk < KCH / 2; kk++)
#pragma unroll
                        for (int q = 0; q < XF_QZ; q++)
                            tc_mma(acc + (uint32_t)q * SCOLS,
                                   a0 + ((((q + sz) * XF_GY + sy) * XF_GX * 16 + kk * 2 * XF_PLANE) >> 4),
                                   b0 + (((u * KCH + kk * 2) * WGRP) >> 4), idesc, (u | kk) != 0);
                }
                asm volatile(
                    "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mma(b)));
                committed = it + 1;
            }
            if (committed > 0)
                mbar_wait(mma((committed - 1) & 1), (uint32_t)((committed - 1) >> 1) & 1u, kConvWaitPolls);
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) {  // box producer
            int issued = 0;
            for (int it = 0; it < ntile; it++) {
                const int b = it & 1;
                if (it >= 2 && !mbar_wait(mma(b), (uint32_t)((it >> 1) - 1) & 1u, kConvWaitPolls)) {
                    failed = true;
                    break;
                }
                int x0, y0, z0;
                origin(first + it * stride, x0, y0, z0);
                const uint32_t dst = xbase0 + b * XBYTES, bar = full(b);
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar),
                             "r"((uint32_t)(KCH * XF_GVOX * 16)));
#pragma unroll
                for (int c = 0; c < KCH; c++)
                    asm volatile(
                        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, "
                        "{%2, %3, %4, %5}], [%6];\n" ::"r"(dst + c * XF_PLANE),
                        "l"(reinterpret_cast<uint64_t>(&tmap)), "r"(c * 8), "r"(x0 - 1), "r"(y0 - 1), "r"(z0 - 1),
                        "r"(bar)
                        : "memory");
                issued = it + 1;
            }
            for (int j = issued - 2; j < issued; j++)
                if (j >= 0) mbar_wait(full(j & 1), (uint32_t)(j >> 1) & 1u, kConvWaitPolls);
        }
        __syncwarp();
    } else {  // epilogue: warps 2..5
        const int quarter = warp & 3;
        const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16);
        float bsh[COUT];
#pragma unroll
        for (int c = 0; c < COUT; c++) bsh[c] = MODE == 2 ? 0.f : (MODE == 1 && c > 0 ? 0.f : bias[c]);
        const int r = quarter * 32 + lane, rx = r & 15, ry = r >> 4;
        for (int it = 0; it < ntile; it++) {
            const int b = it & 1;
            if (!mbar_wait(mma(b), (uint32_t)(it >> 1) & 1u, kConvWaitPolls)) {
                failed = true;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n");
            int x0, y0, z0;
            origin(first + it * stride, x0, y0, z0);
            const int gx = x0 + rx, gy = y0 + ry;
#pragma unroll 1
            for (int zq = 0; zq < XF_QZ; zq++) {
                uint32_t p0[COUT], p1[COUT], p2[COUT];
                const uint32_t col = taddr + (uint32_t)b * ACC_COLS + (uint32_t)zq * SCOLS;
                tmem_ld<COUT>(col, p0);
                tmem_ld<COUT>(col + COUT, p1);
                tmem_ld<COUT>(col + 2 * COUT, p2);
                tmem_wait();
                if (zq == XF_QZ - 1) {  // the accumulator set is read: hand it back
                    asm volatile("tcgen05.fence::before_thread_sync;\n");
                    __syncwarp();
                    if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(fre(b)) : "memory");
                }
                float acc[COUT];
#pragma unroll
                for (int c = 0; c < COUT; c++)  // rows r+1 and r+2 are lanes lane+1, lane+2 (same x-line)
                    acc[c] = __uint_as_float(p0[c]) + __shfl_down_sync(0xffffffffu, __uint_as_float(p1[c]), 1) +
                             __shfl_down_sync(0xffffffffu, __uint_as_float(p2[c]), 2);
                const int gz = z0 + zq;
                if (rx < XF_TX && gx < d.W && gy < d.H && gz < d.D) {
                    const i64 v = gx + (i64)gy * d.W + (i64)gz * d.W * d.H;
                    if constexpr (MODE == 1) {
                        reinterpret_cast<float *>(out)[v] = acc[0] + bsh[0];
                    } else {
                        uint4 *o = reinterpret_cast<uint4 *>(reinterpret_cast<bf16 *>(out) + v * COUT);
                        const uint4 *ax = MODE == 2 ? reinterpret_cast<const uint4 *>(aux + v * COUT) : nullptr;
#pragma unroll
                        for (int q = 0; q < COUT / 8; q++) {
                            uint4 mk = make_uint4(0, 0, 0, 0);
                            if constexpr (MODE == 2) mk = ax[q];
                            const bf16 *mb = reinterpret_cast<const bf16 *>(&mk);
                            uint4 pk;
                            __nv_bfloat162 *p2h = reinterpret_cast<__nv_bfloat162 *>(&pk);
#pragma unroll
                            for (int h = 0; h < 4; h++) {
                                const int ch = q * 8 + 2 * h;
                                float v0 = acc[ch], v1 = acc[ch + 1];
                                if constexpr (MODE == 0) {
                                    v0 = fmaxf(v0 + bsh[ch], 0.f);
                                    v1 = fmaxf(v1 + bsh[ch + 1], 0.f);
                                } else {
                                    if (!(__bfloat162float(mb[2 * h]) > 0.f)) v0 = 0.f;
                                    if (!(__bfloat162float(mb[2 * h + 1]) > 0.f)) v1 = 0.f;
                                }
                                p2h[h] = __floats2bfloat162_rn(v0, v1);
                            }
                            o[q] = pk;
                        }
                    }
                }
            }
        }
    }
    if (failed) atomicOr(err, 1);
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "n"(ALLOC));
}

// The tensor pipe's own ceiling for one instruction shape: one block per SM
// issues `reps` x 8 back-to-back tcgen05.mma of M = 128, N (32, 48, 64, 96,
// 128 or 256), K = 16 (bf16, f32 accumulators) on zeroed shared-memory
// operands, into the accumulators that fit 256 columns in turn, and waits for
// them (bounded).  A convolution made of
// N = 32 products (32 output channels) cannot run faster than this kernel at
// N = 32; measured on GB300 the rate grows with N up to N = 128.
// operands: A (4 KB) at 0, B (N x 32 bytes, <= 8 KB) at 16 KB; the launch asks
// for more shared memory than two blocks can share, so each SM runs one
constexpr uint32_t kRateOperands = 24 * 1024, kRateSmem = 120 * 1024;
template <int N>
__global__ void __launch_bounds__(128, 1) k_mma_rate(int reps, int *err) {
    extern __shared__ __align__(128) unsigned char rs[];
    __shared__ uint32_t tmem_slot;
    __shared__ __align__(8) uint64_t mbar;
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int i = tid; i < (int)(kRateOperands / 4); i += blockDim.x) reinterpret_cast<uint32_t *>(rs)[i] = 0u;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;\n" ::"r"(smem_addr(&tmem_slot)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    const uint32_t bar = smem_addr(&mbar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar));
        asm volatile("fence.mbarrier_init.release.cluster;\n");
    }
    asm volatile("fence.proxy.async.shared::cta;\n");
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    const uint32_t tmem = tmem_slot;
    if (tid == 0) {
        const uint32_t base = smem_addr(rs);
        const uint64_t a = smem_desc(base, 2048, 128), b = smem_desc(base + 16384, N * 16, 128);
        const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | (8u << 24);
        // accumulators side by side in the 256 columns, each at a multiple of
        // the power of two >= N (as the convolutions place theirs)
        constexpr int step = N <= 32 ? 32 : N <= 64 ? 64 : N <= 128 ? 128 : 256, nacc = 256 / step;
        for (int r = 0; r < reps; r++)
#pragma unroll
            for (int q = 0; q < 8; q++) tc_mma(tmem + (uint32_t)((q % nacc) * step), a, b, idesc, (r | q) != 0);
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar));
        if (!mbar_wait(bar, 0u, 1 << 24)) atomicOr(err, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n");
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;\n" ::"r"(tmem));
}

// ------------------------------------------------------------ weight gradient
// dW[tap][n][c] = sum_v dz[v][n] * act[v + off(tap)][c]; db[n] = sum_v dz[v][n].
// GEMM per tap with M = n, N = c, K = vertices of the tile.  Both operands are
// read transposed from the channels-last tiles by ldmatrix.trans.  16 warps
// share the 27 x (COUT/16) (tap, m-tile) units; each keeps its units'
// accumulators in registers across all tiles of the block, and the block
// writes one partial sum of every parameter of the layer to part[blockIdx.x].
template <int CIN, int COUT>
__global__ void __launch_bounds__(512, 1) k_wgrad(Dims d, const bf16 *__restrict__ act, const bf16 *__restrict__ dz,
                                                  float *__restrict__ part) {
    constexpr int AP = CIN + 8, DP = COUT + 8, NT = CIN / 8, MT = COUT / 16, UNITS = 27 * MT, NW = 16;
    constexpr int UPW = (UNITS + NW - 1) / NW;
    constexpr i64 NPAR = 27LL * COUT * CIN + COUT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    bf16 *as0 = reinterpret_cast<bf16 *>(smem_raw);  // 2 x [HALO][AP]
    bf16 *ds0 = as0 + 2 * HALO * AP;                  // 2 x [TV][DP]
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
    float acc[UPW][NT][4];
#pragma unroll
    for (int u = 0; u < UPW; u++)
#pragma unroll
        for (int n = 0; n < NT; n++)
#pragma unroll
            for (int k = 0; k < 4; k++) acc[u][n][k] = 0.f;
    float bacc = 0.f;
    // ldmatrix.trans roles.  A (dz^T: rows = out channel, k = vertex): lane
    // gives vertex (lane&7) + 8*(lane>>4), channel block 8*((lane>>3)&1).
    // B (act: k = vertex, n = in channel): vertex (lane&7) + 8*((lane>>3)&1),
    // channel block 8*(lane>>4) within a pair of n-tiles.
    const int va = (lane & 7) + 8 * (lane >> 4), ca = 8 * ((lane >> 3) & 1);
    const int vb = (lane & 7) + 8 * ((lane >> 3) & 1), cb = 8 * (lane >> 4);

    i64 tile = blockIdx.x;
    int buf = 0;
    if (tile < d.ntiles) {
        int x0, y0, z0;
        tile_origin(d, tile, x0, y0, z0);
        load_box<CIN, HX, HY, HZ>(as0, act, d, x0 - 1, y0 - 1, z0 - 1);
        load_box<COUT, TX, TY, TZ>(ds0, dz, d, x0, y0, z0);
    }
    cp_commit();
    for (; tile < d.ntiles; tile += gridDim.x, buf ^= 1) {
        const i64 next = tile + gridDim.x;
        if (next < d.ntiles) {
            int x0, y0, z0;
            tile_origin(d, next, x0, y0, z0);
            load_box<CIN, HX, HY, HZ>(as0 + (buf ^ 1) * HALO * AP, act, d, x0 - 1, y0 - 1, z0 - 1);
            load_box<COUT, TX, TY, TZ>(ds0 + (buf ^ 1) * TV * DP, dz, d, x0, y0, z0);
        }
        cp_commit();
        cp_wait<1>();
        __syncthreads();
        const bf16 *as = as0 + buf * HALO * AP, *ds = ds0 + buf * TV * DP;
        if (lane < COUT)
            for (int v = warp * (TV / NW); v < (warp + 1) * (TV / NW); v++) bacc += __bfloat162float(ds[v * DP + lane]);
#pragma unroll
        for (int u = 0; u < UPW; u++) {
            const int unit = warp + u * NW;
            if (unit >= UNITS) continue;
            const int tap = unit / MT, mt = unit - tap * MT;
            const int dx = tap % 3 - 1, dy = (tap / 3) % 3 - 1, dzz = tap / 9 - 1;
            const int toff = (dzz * HY + dy) * HX + dx;
#pragma unroll 4
            for (int ks = 0; ks < TV / 16; ks++) {
                uint32_t a[4];
                ldm4t(a, ds + (ks * 16 + va) * DP + mt * 16 + ca);
                const int lb = ks * 16 + vb;
                const int hb = (((lb >> 6) + 1) * HY + ((lb >> 3) & 7) + 1) * HX + (lb & 7) + 1 + toff;
#pragma unroll
                for (int nt = 0; nt < NT; nt += 2) {
                    uint32_t b[4];
                    ldm4t(b, as + hb * AP + nt * 8 + cb);
                    mma16816(acc[u][nt], a, b[0], b[1]);
                    mma16816(acc[u][nt + 1], a, b[2], b[3]);
                }
            }
        }
        __syncthreads();
    }
    cp_wait<0>();
    float *p = part + (i64)blockIdx.x * NPAR;
#pragma unroll
    for (int u = 0; u < UPW; u++) {
        const int unit = warp + u * NW;
        if (unit >= UNITS) continue;
        const int tap = unit / MT, mt = unit - tap * MT;
#pragma unroll
        for (int nt = 0; nt < NT; nt++) {
            const int n0 = mt * 16 + g, c0 = nt * 8 + 2 * t;
            float *q = p + ((i64)tap * COUT + n0) * CIN + c0;
            q[0] = acc[u][nt][0];
            q[1] = acc[u][nt][1];
            q[8 * CIN] = acc[u][nt][2];
            q[8 * CIN + 1] = acc[u][nt][3];
        }
    }
    // bias: fixed-order sum of the 16 warps' partials
    __syncthreads();
    float *red = reinterpret_cast<float *>(smem_raw);
    if (lane < COUT) red[warp * COUT + lane] = bacc;
    __syncthreads();
    if (tid < COUT) {
        float s = 0.f;
        for (int w = 0; w < NW; w++) s += red[w * COUT + tid];
        p[27LL * COUT * CIN + tid] = s;
    }
}

// grad[i] = scale * sum over blocks (in block order) of part[b][i]
__global__ void k_reduce(const float *__restrict__ part, int nblk, i64 n, const float *__restrict__ scale,
                         float *__restrict__ grad) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int b = 0; b < nblk; b++) s += part[(i64)b * n + i];
        grad[i] = s * *scale;
    }
}

// ------------------------------------------------------------------- the loss
// Weighted over vertices (weight = the byte active[v], 0 = ignored):
// L = sum w (tanh(o) - target)^2 / sum w.  Writes dL/do without the 1/sum w
// factor (applied by k_reduce) into channel 0 of dz (16 channels, the others
// 0), and per-block (weighted sum, sum of weights) partials.
constexpr int kLossBlocks = 1024;
__global__ void k_loss(i64 V, const float *__restrict__ o, const float *__restrict__ target,
                       const uint8_t *__restrict__ active, bf16 *__restrict__ dz, double *__restrict__ part) {
    double ls = 0.0, cnt = 0.0;
    for (i64 v = (i64)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (i64)gridDim.x * blockDim.x) {
        float gval = 0.f;
        const float w = (float)active[v];
        if (w > 0.f) {
            const float y = tanhf(o[v]);
            const float e = y - target[v];
            ls += (double)w * e * e;
            cnt += w;
            gval = 2.f * w * e * (1.f - y * y);
        }
        const __nv_bfloat162 lo = __floats2bfloat162_rn(gval, 0.f);
        uint4 first = make_uint4(*reinterpret_cast<const uint32_t *>(&lo), 0u, 0u, 0u);
        reinterpret_cast<uint4 *>(dz + v * 16)[0] = first;
        reinterpret_cast<uint4 *>(dz + v * 16)[1] = make_uint4(0u, 0u, 0u, 0u);
    }
    __shared__ double sl[32], sc[32];
    for (int off = 16; off > 0; off >>= 1) {
        ls += __shfl_down_sync(0xffffffffu, ls, off);
        cnt += __shfl_down_sync(0xffffffffu, cnt, off);
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        sl[w] = ls;
        sc[w] = cnt;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) {
            a += sl[i];
            b += sc[i];
        }
        part[2 * blockIdx.x] = a;
        part[2 * blockIdx.x + 1] = b;
    }
}
// res[0] = mean loss, res[1] = sum of weights; scale = 1 / that (0 if none)
__global__ void k_loss_final(const double *__restrict__ part, int nblk, double *__restrict__ res,
                             float *__restrict__ scale) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double a = 0.0, b = 0.0;
    for (int i = 0; i < nblk; i++) {
        a += part[2 * i];
        b += part[2 * i + 1];
    }
    res[0] = b > 0 ? a / b : 0.0;
    res[1] = b;
    *scale = b > 0 ? (float)(1.0 / b) : 0.f;
}

// ------------------------------------------------------------ Adam + weights
__global__ void k_adam(i64 n, float *__restrict__ w, const float *__restrict__ gr, float *__restrict__ m1,
                       float *__restrict__ m2, float lr, float b1, float b2, float eps, float c1, float c2) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        const float gv = gr[i];
        const float a = b1 * m1[i] + (1.f - b1) * gv;
        const float b = b2 * m2[i] + (1.f - b2) * gv * gv;
        m1[i] = a;
        m2[i] = b;
        w[i] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
    }
}
// bf16 copies of one layer's weights: forward [tap][n][c] and transposed
// [tap][c][n] (for the data gradient)
__global__ void k_pack(const float *__restrict__ w, int cin, int cout, bf16 *__restrict__ wf, bf16 *__restrict__ wt) {
    const int n = 27 * cin * cout;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int c = i % cin, no = (i / cin) % cout, tap = i / (cin * cout);
        const bf16 b = __float2bfloat16_rn(w[i]);
        wf[i] = b;
        wt[((i64)tap * cin + c) * cout + no] = b;
    }
}

}  // namespace

// ====================================================================== host
struct dmtz_cnn {
    float min_drop = 0.5f;  // proposal applied only where it lowers g by >= min_drop * bound
    int device = 0;
    int nsm = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    float *w = nullptr, *grad = nullptr, *m1 = nullptr, *m2 = nullptr;  // kParams each
    bf16 *wf = nullptr, *wt = nullptr;  // bf16 weights, forward and transposed, per layer at woff[l]
    float *part = nullptr;              // weight-gradient partials, part_blocks x (largest layer)
    int part_blocks = 0;
    double *lpart = nullptr, *lres = nullptr;
    float *scale = nullptr;
    i64 step = 0;
    // activations of the last forward pass (a[2] aliases a[0] unless kept for training)
    i64 capV = 0;
    bool cap_train = false;
    bf16 *a[3] = {nullptr, nullptr, nullptr};
    bf16 *dz4 = nullptr, *gA = nullptr, *gB = nullptr;
    int lastW = 0, lastH = 0, lastD = 0, last_train = 0;
    const bf16 *last_feat = nullptr;
    const float *last_out = nullptr;
    // convolutions on tcgen05 (1, the default) or on mma.sync (0)
    int tensor_path = 2;
    int *tc_err = nullptr;  // set by a tcgen05 convolution whose wait timed out
    // warm-start scratch
    i64 capS = 0;
    bf16 *feat = nullptr;
    uint8_t *active = nullptr;
    float *out = nullptr;
};

namespace {

i64 woff(int l) {
    i64 o = 0;
    for (int k = 0; k < l; k++) o += 27LL * LCIN[k] * LCOUT[k];
    return o;
}
constexpr i64 kWeights = 27LL * (16 * 32 + 32 * 32 + 32 * 32 + 32 * 16);

dmtz_status nfail(dmtz_cnn *n, dmtz_status s, const std::string &m) {
    if (n) n->err = m;
    return s;
}
#define NCK(call)                                                                                 \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return nfail(net, DMTZ_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <class T>
cudaError_t nalloc(T **p, i64 n) {
    return cudaMalloc((void **)p, sizeof(T) * (size_t)std::max<i64>(n, 1));
}

uint64_t splitmix(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

template <int CIN, int COUT, int MODE, bool FLIP>
constexpr size_t conv_smem() {
    return (size_t)(27 * COUT * (CIN + 8) + 2 * HALO * (CIN + 8)) * sizeof(bf16);
}
template <int CIN, int COUT>
constexpr size_t wgrad_smem() {
    return (size_t)(2 * HALO * (CIN + 8) + 2 * TV * (COUT + 8)) * sizeof(bf16);
}

// launches a persistent kernel with as many blocks as fit on the GPU (at most
// one per tile); the dynamic shared-memory limit is raised once per kernel
template <class K>
dmtz_status launch_persistent(dmtz_cnn *net, K kernel, int threads, size_t smem, i64 ntiles, int cap_blocks,
                              int *used_blocks, cudaStream_t st, void **args) {
    NCK(cudaFuncSetAttribute((const void *)kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    NCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem));
    if (per_sm < 1) return nfail(net, DMTZ_ERR_CUDA, "convolution kernel does not fit on an SM");
    i64 blocks = std::min<i64>(ntiles, (i64)per_sm * net->nsm);
    if (cap_blocks > 0) blocks = std::min<i64>(blocks, cap_blocks);
    blocks = std::max<i64>(blocks, 1);
    if (used_blocks) *used_blocks = (int)blocks;
    NCK(cudaLaunchKernel((const void *)kernel, dim3((unsigned)blocks), dim3(threads), args, smem, st));
    return DMTZ_OK;
}

// tensor map of a channels-last bf16 activation tensor for the TMA boxes of
// k_conv_tc and k_conv_tcx (the CUDA driver's encoder, looked up once through
// the runtime)
dmtz_status box_map(dmtz_cnn *net, CUtensorMap *tm, const bf16 *act, int C, int W, int H, int D, int bx = GX,
                    int by = GY, int bz = GZ) {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        cudaDriverEntryPointQueryResult q;
        void *fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !fn)
            return nfail(net, DMTZ_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    const cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)D};
    const cuuint64_t strides[3] = {(cuuint64_t)C * 2, (cuuint64_t)C * 2 * W, (cuuint64_t)C * 2 * W * H};
    const cuuint32_t box[4] = {8, (cuuint32_t)bx, (cuuint32_t)by, (cuuint32_t)bz}, estr[4] = {1, 1, 1, 1};
    const CUresult r = encode(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16 *>(act), dims, strides, box,
                              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return nfail(net, DMTZ_ERR_CUDA, "cuTensorMapEncodeTiled failed");
    return DMTZ_OK;
}

template <int CIN, int COUT, int MODE, bool FLIP>
dmtz_status conv(dmtz_cnn *net, const Dims &d, const bf16 *in, const bf16 *w, const float *bias, void *out,
                 const bf16 *aux, cudaStream_t st) {
    if (net->tensor_path == 2) {
        Dims dt = make_xf_dims(d.W, d.H, d.D);
        CUtensorMap tm;
        dmtz_status s = box_map(net, &tm, in, CIN, d.W, d.H, d.D, XF_GX, XF_GY, XF_GZ);
        if (s != DMTZ_OK) return s;
        int *err = net->tc_err;
        void *args[] = {&tm, &dt, &w, &bias, &out, &aux, &err};
        // each block holds 2 x 2 x 64 or 2 x 2 x 128 tensor-memory columns; no more blocks per SM
        // than the 512 columns hold (a second block's allocation would wait for the first to exit)
        const int cap = net->nsm * (int)(512 / (4 * xf_cols<COUT>()));
        return launch_persistent(net, k_conv_tcx<CIN, COUT, MODE, FLIP>, kConvThreads, xf_smem<CIN, COUT>(),
                                 dt.ntiles, cap, nullptr, st, args);
    }
    if (net->tensor_path) {
        Dims dt = make_tc_dims(d.W, d.H, d.D);
        CUtensorMap tm;
        dmtz_status s = box_map(net, &tm, in, CIN, d.W, d.H, d.D);
        if (s != DMTZ_OK) return s;
        int *err = net->tc_err;
        void *args[] = {&tm, &dt, &w, &bias, &out, &aux, &err};
        return launch_persistent(net, k_conv_tc<CIN, COUT, MODE, FLIP>, kConvThreads, tc_smem<CIN, COUT>(), dt.ntiles, 0,
                                 nullptr, st, args);
    }
    Dims dd = d;
    void *args[] = {&dd, &in, &w, &bias, &out, &aux};
    return launch_persistent(net, k_conv<CIN, COUT, MODE, FLIP>, 256, conv_smem<CIN, COUT, MODE, FLIP>(), d.ntiles, 0,
                             nullptr, st, args);
}

template <int CIN, int COUT>
dmtz_status wgrad(dmtz_cnn *net, const Dims &d, const bf16 *act, const bf16 *dz, float *grad_out, cudaStream_t st) {
    Dims dd = d;
    float *part = net->part;
    void *args[] = {&dd, &act, &dz, &part};
    int used = 0;
    dmtz_status s = launch_persistent(net, k_wgrad<CIN, COUT>, 512, wgrad_smem<CIN, COUT>(), d.ntiles,
                                      net->part_blocks, &used, st, args);
    if (s != DMTZ_OK) return s;
    const i64 n = 27LL * COUT * CIN + COUT;
    k_reduce<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(net->part, used, n, net->scale, grad_out);
    NCK(cudaGetLastError());
    return DMTZ_OK;
}

dmtz_status pack(dmtz_cnn *net, cudaStream_t st) {
    for (int l = 0; l < NLAYER; l++) {
        k_pack<<<64, 256, 0, st>>>(net->w + layer_offset(l), LCIN[l], LCOUT[l], net->wf + woff(l), net->wt + woff(l));
    }
    NCK(cudaGetLastError());
    return DMTZ_OK;
}

dmtz_status ensure_act(dmtz_cnn *net, i64 V, bool train) {
    if (V <= net->capV && (!train || net->cap_train)) return DMTZ_OK;
    cudaFree(net->a[0]);
    cudaFree(net->a[1]);
    if (net->cap_train) cudaFree(net->a[2]);
    cudaFree(net->dz4);
    cudaFree(net->gA);
    cudaFree(net->gB);
    net->a[0] = net->a[1] = net->a[2] = net->dz4 = net->gA = net->gB = nullptr;
    net->capV = 0;
    net->cap_train = false;
    const i64 cap = std::max(V, net->capV);
    NCK(nalloc(&net->a[0], cap * 32));
    NCK(nalloc(&net->a[1], cap * 32));
    if (train) {
        NCK(nalloc(&net->a[2], cap * 32));
        NCK(nalloc(&net->dz4, cap * 16));
        NCK(nalloc(&net->gA, cap * 32));
        NCK(nalloc(&net->gB, cap * 32));
    } else {
        net->a[2] = net->a[0];
    }
    net->capV = cap;
    net->cap_train = train;
    return DMTZ_OK;
}

dmtz_status check_grid(dmtz_cnn *net, int W, int H, int D) {
    if (!net) return DMTZ_ERR_ARG;
    if (W < 1 || H < 1 || D < 1) return nfail(net, DMTZ_ERR_ARG, "grid dimensions must be >= 1");
    if ((i64)W * H * D > (1LL << 40)) return nfail(net, DMTZ_ERR_ARG, "grid too large");
    return DMTZ_OK;
}

}  // namespace

namespace dmtz_cnn_impl {

const std::string &error_of(const dmtz_cnn *net) { return net->err; }
int device_of(const dmtz_cnn *net) { return net->device; }
float min_drop_of(const dmtz_cnn *net) { return net->min_drop; }

dmtz_status forward_on(dmtz_cnn *net, int W, int H, int D, const bf16 *feat, float *out, int train,
                       cudaStream_t st) {
    dmtz_status s = check_grid(net, W, H, D);
    if (s != DMTZ_OK) return s;
    if (!feat || !out || ((uintptr_t)feat & 15)) return nfail(net, DMTZ_ERR_ARG, "features must be 16-byte aligned");
    NCK(cudaSetDevice(net->device));
    const Dims d = make_dims(W, H, D);
    const i64 V = (i64)W * H * D;
    if ((s = ensure_act(net, V, train != 0)) != DMTZ_OK) return s;
    bf16 *a1 = net->a[0], *a2 = net->a[1], *a3 = net->a[2];
    const float *w = net->w;
    if ((s = conv<16, 32, 0, false>(net, d, feat, net->wf + woff(0), w + layer_offset(0) + 27 * 32 * 16, a1, nullptr,
                                    st)) != DMTZ_OK)
        return s;
    if ((s = conv<32, 32, 0, false>(net, d, a1, net->wf + woff(1), w + layer_offset(1) + 27 * 32 * 32, a2, nullptr,
                                    st)) != DMTZ_OK)
        return s;
    if ((s = conv<32, 32, 0, false>(net, d, a2, net->wf + woff(2), w + layer_offset(2) + 27 * 32 * 32, a3, nullptr,
                                    st)) != DMTZ_OK)
        return s;
    if ((s = conv<32, 16, 1, false>(net, d, a3, net->wf + woff(3), w + layer_offset(3) + 27 * 16 * 32, out, nullptr,
                                    st)) != DMTZ_OK)
        return s;
    net->lastW = W;
    net->lastH = H;
    net->lastD = D;
    net->last_train = train != 0;
    net->last_feat = feat;
    net->last_out = out;
    return DMTZ_OK;
}

dmtz_status scratch(dmtz_cnn *net, int64_t V, bf16 **feat, uint8_t **active, float **out) {
    if (V > net->capS) {
        cudaFree(net->feat);
        cudaFree(net->active);
        cudaFree(net->out);
        net->feat = nullptr;
        net->active = nullptr;
        net->out = nullptr;
        net->capS = 0;
        NCK(nalloc(&net->feat, V * kFeat));
        NCK(nalloc(&net->active, V));
        NCK(nalloc(&net->out, V));
        net->capS = V;
    }
    *feat = net->feat;
    *active = net->active;
    *out = net->out;
    return DMTZ_OK;
}

}  // namespace dmtz_cnn_impl

using dmtz_cnn_impl::forward_on;

extern "C" {

int64_t dmtz_cnn_num_params(void) { return kParams; }

dmtz_status dmtz_cnn_create(dmtz_cnn **out, int device, uint64_t seed) {
    if (!out) return DMTZ_ERR_ARG;
    *out = nullptr;
    dmtz_cnn *net = new dmtz_cnn();
    net->device = device;
    auto bail = [&](dmtz_status s) {
        dmtz_cnn_destroy(net);
        return s;
    };
    if (cudaSetDevice(device) != cudaSuccess) return bail(DMTZ_ERR_CUDA);
    if (cudaDeviceGetAttribute(&net->nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return bail(DMTZ_ERR_CUDA);
    if (cudaStreamCreateWithFlags(&net->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(DMTZ_ERR_CUDA);
    net->part_blocks = 2 * net->nsm;
    i64 largest = 0;
    for (int l = 0; l < NLAYER; l++) largest = std::max(largest, layer_params(l));
    if (nalloc(&net->w, kParams) || nalloc(&net->grad, kParams) || nalloc(&net->m1, kParams) ||
        nalloc(&net->m2, kParams) || nalloc(&net->wf, kWeights) || nalloc(&net->wt, kWeights) ||
        nalloc(&net->part, (i64)net->part_blocks * largest) || nalloc(&net->lpart, 2 * kLossBlocks) ||
        nalloc(&net->lres, 2) || nalloc(&net->scale, 1) || nalloc(&net->tc_err, 1))
        return bail(DMTZ_ERR_CUDA);
    if (cudaMemset(net->tc_err, 0, sizeof(int)) != cudaSuccess) return bail(DMTZ_ERR_CUDA);
    // He-uniform weights (bound sqrt(6 / fan_in)); the output layer 0.1x and
    // only its channel 0 nonzero; zero biases
    std::vector<float> h((size_t)kParams, 0.f);
    uint64_t s = seed ^ 0x6A09E667F3BCC909ull;
    for (int l = 0; l < NLAYER; l++) {
        const double b = std::sqrt(6.0 / (27.0 * LCIN[l])) * (l == NLAYER - 1 ? 0.1 : 1.0);
        float *p = h.data() + layer_offset(l);
        for (int tap = 0; tap < 27; tap++)
            for (int n = 0; n < LCOUT[l]; n++)
                for (int c = 0; c < LCIN[l]; c++) {
                    const double u = (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0);
                    const bool live = l < NLAYER - 1 || n == 0;
                    p[((i64)tap * LCOUT[l] + n) * LCIN[l] + c] = live ? (float)((2.0 * u - 1.0) * b) : 0.f;
                }
    }
    if (dmtz_cnn_set_params(net, h.data()) != DMTZ_OK) return bail(DMTZ_ERR_CUDA);
    *out = net;
    return DMTZ_OK;
}

void dmtz_cnn_destroy(dmtz_cnn *net) {
    if (!net) return;
    cudaSetDevice(net->device);
    if (net->stream) cudaStreamSynchronize(net->stream);
    for (void *p : {(void *)net->w, (void *)net->grad, (void *)net->m1, (void *)net->m2, (void *)net->wf,
                    (void *)net->wt, (void *)net->part, (void *)net->lpart, (void *)net->lres, (void *)net->scale,
                    (void *)net->a[0], (void *)net->a[1], (void *)net->dz4, (void *)net->gA, (void *)net->gB,
                    (void *)net->feat, (void *)net->active, (void *)net->out, (void *)net->tc_err})
        cudaFree(p);
    if (net->cap_train) cudaFree(net->a[2]);
    if (net->stream) cudaStreamDestroy(net->stream);
    delete net;
}

const char *dmtz_cnn_last_error(const dmtz_cnn *net) { return net ? net->err.c_str() : "null network"; }

dmtz_status dmtz_cnn_set_min_drop(dmtz_cnn *net, float min_drop) {
    if (!net) return DMTZ_ERR_ARG;
    if (!(min_drop >= 0.f) || !(min_drop <= 2.f)) return nfail(net, DMTZ_ERR_ARG, "min_drop must be in [0, 2]");
    net->min_drop = min_drop;
    return DMTZ_OK;
}

dmtz_status dmtz_cnn_set_params(dmtz_cnn *net, const float *host) {
    if (!net || !host) return DMTZ_ERR_ARG;
    NCK(cudaSetDevice(net->device));
    NCK(cudaMemcpyAsync(net->w, host, sizeof(float) * kParams, cudaMemcpyHostToDevice, net->stream));
    NCK(cudaMemsetAsync(net->m1, 0, sizeof(float) * kParams, net->stream));
    NCK(cudaMemsetAsync(net->m2, 0, sizeof(float) * kParams, net->stream));
    NCK(cudaMemsetAsync(net->grad, 0, sizeof(float) * kParams, net->stream));
    net->step = 0;
    dmtz_status s = pack(net, net->stream);
    if (s != DMTZ_OK) return s;
    NCK(cudaStreamSynchronize(net->stream));
    return DMTZ_OK;
}

dmtz_status dmtz_cnn_get_params(dmtz_cnn *net, float *host) {
    if (!net || !host) return DMTZ_ERR_ARG;
    NCK(cudaSetDevice(net->device));
    NCK(cudaMemcpyAsync(host, net->w, sizeof(float) * kParams, cudaMemcpyDeviceToHost, net->stream));
    NCK(cudaStreamSynchronize(net->stream));
    return DMTZ_OK;
}

dmtz_status dmtz_cnn_get_grads(dmtz_cnn *net, float *host) {
    if (!net || !host) return DMTZ_ERR_ARG;
    NCK(cudaSetDevice(net->device));
    NCK(cudaMemcpyAsync(host, net->grad, sizeof(float) * kParams, cudaMemcpyDeviceToHost, net->stream));
    NCK(cudaStreamSynchronize(net->stream));
    return DMTZ_OK;
}

// a tcgen05 convolution whose completion wait timed out leaves a flag (the
// kernel itself returns); the synchronous calls report it
static dmtz_status check_tc(dmtz_cnn *net) {
    int e = 0;
    NCK(cudaMemcpy(&e, net->tc_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
        NCK(cudaMemset(net->tc_err, 0, sizeof(int)));
        return nfail(net, DMTZ_ERR_CUDA, "a tensor-core convolution timed out waiting for its MMAs");
    }
    return DMTZ_OK;
}

dmtz_status dmtz_cnn_set_tensor_path(dmtz_cnn *net, int path) {
    if (!net || path < 0 || path > 2) return DMTZ_ERR_ARG;
    net->tensor_path = path;
    return DMTZ_OK;
}

dmtz_status dmtz_cnn_mma_ceiling(dmtz_cnn *net, int n, int reps, double *tflops) {
    // the shapes are compile-time constants: the issuing thread does no arithmetic between MMAs
    void (*kern)(int, int *) = n == 32 ? k_mma_rate<32> : n == 48 ? k_mma_rate<48> : n == 64 ? k_mma_rate<64>
                             : n == 96 ? k_mma_rate<96> : n == 128 ? k_mma_rate<128> : n == 256 ? k_mma_rate<256>
                                                                                                 : nullptr;
    if (!net || !tflops || reps < 1 || reps > (1 << 16) || !kern) return DMTZ_ERR_ARG;
    NCK(cudaSetDevice(net->device));
    cudaStream_t st = net->stream;
    NCK(cudaFuncSetAttribute((const void *)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRateSmem));
    int *err = nullptr;
    NCK(cudaMalloc(&err, sizeof(int)));
    cudaEvent_t e[2];
    cudaEventCreate(&e[0]);
    cudaEventCreate(&e[1]);
    cudaMemsetAsync(err, 0, sizeof(int), st);
    kern<<<net->nsm, 128, kRateSmem, st>>>(reps, err);  // warm-up
    cudaEventRecord(e[0], st);
    kern<<<net->nsm, 128, kRateSmem, st>>>(reps, err);
    cudaEventRecord(e[1], st);
    int herr = 0;
    cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st);
    const cudaError_t ce = cudaStreamSynchronize(st);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e[0], e[1]);
    cudaEventDestroy(e[0]);
    cudaEventDestroy(e[1]);
    cudaFree(err);
    if (ce != cudaSuccess) return nfail(net, DMTZ_ERR_CUDA, std::string("k_mma_rate: ") + cudaGetErrorString(ce));
    if (herr) return nfail(net, DMTZ_ERR_CUDA, "k_mma_rate: the MMAs did not complete in time");
    *tflops = 2.0 * 128 * n * 16 * 8.0 * reps * net->nsm / (ms * 1e-3) / 1e12;
    return DMTZ_OK;
}

dmtz_status dmtz_cnn_forward(dmtz_cnn *net, int W, int H, int D, const void *feat, float *out, int train) {
    if (!net) return DMTZ_ERR_ARG;
    dmtz_status s = forward_on(net, W, H, D, static_cast<const bf16 *>(feat), out, train, net->stream);
    if (s != DMTZ_OK) return s;
    NCK(cudaStreamSynchronize(net->stream));
    return check_tc(net);
}

dmtz_status dmtz_cnn_backward(dmtz_cnn *net, int W, int H, int D, const float *target, const uint8_t *active,
                              double *loss) {
    dmtz_status s = check_grid(net, W, H, D);
    if (s != DMTZ_OK) return s;
    if (!target || !active) return nfail(net, DMTZ_ERR_ARG, "null target or mask");
    if (!net->last_train || net->lastW != W || net->lastH != H || net->lastD != D)
        return nfail(net, DMTZ_ERR_ARG, "backward needs a training forward pass on the same grid");
    NCK(cudaSetDevice(net->device));
    cudaStream_t st = net->stream;
    const Dims d = make_dims(W, H, D);
    const i64 V = (i64)W * H * D;
    k_loss<<<kLossBlocks, 256, 0, st>>>(V, net->last_out, target, active, net->dz4, net->lpart);
    k_loss_final<<<1, 32, 0, st>>>(net->lpart, kLossBlocks, net->lres, net->scale);
    NCK(cudaGetLastError());
    bf16 *a1 = net->a[0], *a2 = net->a[1], *a3 = net->a[2];
    float *gr = net->grad;
    // layer 4: data gradient into a3's space (ReLU mask of a3), weight gradient
    if ((s = conv<16, 32, 2, true>(net, d, net->dz4, net->wt + woff(3), nullptr, net->gA, a3, st)) != DMTZ_OK) return s;
    if ((s = wgrad<32, 16>(net, d, a3, net->dz4, gr + layer_offset(3), st)) != DMTZ_OK) return s;
    // layer 3
    if ((s = conv<32, 32, 2, true>(net, d, net->gA, net->wt + woff(2), nullptr, net->gB, a2, st)) != DMTZ_OK) return s;
    if ((s = wgrad<32, 32>(net, d, a2, net->gA, gr + layer_offset(2), st)) != DMTZ_OK) return s;
    // layer 2
    if ((s = conv<32, 32, 2, true>(net, d, net->gB, net->wt + woff(1), nullptr, net->gA, a1, st)) != DMTZ_OK) return s;
    if ((s = wgrad<32, 32>(net, d, a1, net->gB, gr + layer_offset(1), st)) != DMTZ_OK) return s;
    // layer 1 (no data gradient of the features)
    if ((s = wgrad<16, 32>(net, d, net->last_feat, net->gA, gr + layer_offset(0), st)) != DMTZ_OK) return s;
    double res[2] = {0, 0};
    NCK(cudaMemcpyAsync(res, net->lres, sizeof(res), cudaMemcpyDeviceToHost, st));
    NCK(cudaStreamSynchronize(st));
    if (loss) *loss = res[0];
    return check_tc(net);
}

dmtz_status dmtz_cnn_step(dmtz_cnn *net, float lr) {
    if (!net) return DMTZ_ERR_ARG;
    if (!(lr >= 0.f) || !std::isfinite(lr)) return nfail(net, DMTZ_ERR_ARG, "learning rate must be finite, >= 0");
    NCK(cudaSetDevice(net->device));
    net->step++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = (float)(1.0 - std::pow((double)b1, (double)net->step));
    const float c2 = (float)(1.0 - std::pow((double)b2, (double)net->step));
    k_adam<<<(unsigned)((kParams + 255) / 256), 256, 0, net->stream>>>(kParams, net->w, net->grad, net->m1, net->m2,
                                                                       lr, b1, b2, 1e-8f, c1, c2);
    NCK(cudaGetLastError());
    dmtz_status s = pack(net, net->stream);
    if (s != DMTZ_OK) return s;
    NCK(cudaStreamSynchronize(net->stream));
    return DMTZ_OK;
}

}  // extern "C"

extern "C" dmtz_status dmtz_cnn_profile(dmtz_cnn *net, int W, int H, int D, const void *feat, float *out,
                                        const float *target, const uint8_t *active, int reps, double ms[4]) {
    dmtz_status s = check_grid(net, W, H, D);
    if (s != DMTZ_OK) return s;
    if (!ms || reps < 1 || !target || !active) return nfail(net, DMTZ_ERR_ARG, "bad profile arguments");
    NCK(cudaSetDevice(net->device));
    cudaStream_t st = net->stream;
    const bf16 *fb = static_cast<const bf16 *>(feat);
    cudaEvent_t e[2];
    NCK(cudaEventCreate(&e[0]));
    NCK(cudaEventCreate(&e[1]));
    float t = 0.f;
    auto timed = [&](auto &&body, double &acc) -> dmtz_status {
        NCK(cudaEventRecord(e[0], st));
        for (int r = 0; r < reps; r++) {
            dmtz_status q = body();
            if (q != DMTZ_OK) return q;
        }
        NCK(cudaEventRecord(e[1], st));
        NCK(cudaEventSynchronize(e[1]));
        NCK(cudaEventElapsedTime(&t, e[0], e[1]));
        acc = (double)t / reps;
        return DMTZ_OK;
    };
    // the training steps are undone afterwards: weights, Adam moments and step count
    float *keep = nullptr;
    NCK(nalloc(&keep, 3 * kParams));
    NCK(cudaMemcpyAsync(keep, net->w, sizeof(float) * kParams, cudaMemcpyDeviceToDevice, st));
    NCK(cudaMemcpyAsync(keep + kParams, net->m1, sizeof(float) * kParams, cudaMemcpyDeviceToDevice, st));
    NCK(cudaMemcpyAsync(keep + 2 * kParams, net->m2, sizeof(float) * kParams, cudaMemcpyDeviceToDevice, st));
    const i64 step0 = net->step;
    const Dims d = make_dims(W, H, D);
    if ((s = forward_on(net, W, H, D, fb, out, 1, st)) != DMTZ_OK) return s;  // warm-up, sizes buffers
    NCK(cudaStreamSynchronize(st));
    s = timed([&]() { return forward_on(net, W, H, D, fb, out, 0, st); }, ms[0]);
    if (s == DMTZ_OK)
        s = timed(
            [&]() {
                dmtz_status q = forward_on(net, W, H, D, fb, out, 1, st);
                if (q == DMTZ_OK) q = dmtz_cnn_backward(net, W, H, D, target, active, nullptr);
                if (q == DMTZ_OK) q = dmtz_cnn_step(net, 0.f);
                return q;
            },
            ms[1]);
    if (s == DMTZ_OK)
        s = timed(
            [&]() {
                return conv<32, 32, 0, false>(net, d, net->a[0], net->wf + woff(1),
                                              net->w + layer_offset(1) + 27 * 32 * 32, net->a[1], nullptr, st);
            },
            ms[2]);
    if (s == DMTZ_OK)
        s = timed([&]() { return wgrad<32, 32>(net, d, net->a[1], net->gB, net->grad + layer_offset(2), st); },
                  ms[3]);
    cudaEventDestroy(e[0]);
    cudaEventDestroy(e[1]);
    cudaMemcpyAsync(net->w, keep, sizeof(float) * kParams, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(net->m1, keep + kParams, sizeof(float) * kParams, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(net->m2, keep + 2 * kParams, sizeof(float) * kParams, cudaMemcpyDeviceToDevice, st);
    net->step = step0;
    const dmtz_status sp = pack(net, st);
    NCK(cudaStreamSynchronize(st));
    cudaFree(keep);
    return s != DMTZ_OK ? s : sp;
}
