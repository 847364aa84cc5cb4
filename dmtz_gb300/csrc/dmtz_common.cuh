// dmtz_common.cuh — grid geometry, order keys, reference cell numbering and
// the packed per-anchor gradient state shared by all kernels.
//
// Cells are owned by an anchor vertex (the minimum corner of the cell's
// bounding box): 1 vertex, 7 edge families, 12 triangle slots, 6 tetrahedron
// slots (see gen_topology.py).  The discrete gradient of a field is stored per
// anchor as:
//   pv  (u8)  : steepest-descent direction 0..13 of the vertex, 15 = none
//               (processVertices, main_3d.cu:1930-1988)
//   eup (u32) : 7 x 3 bits, edge -> triangle pairing, coface index + 1
//   fup (u32) : 12 x 2 bits, triangle -> tetrahedron pairing, coface index + 1
// The reference's union-valued arrays paired_vertices / _edges / _faces /
// _tetrahedras are reconstructed from these on demand (pv_ref, pe_ref, pf_ref,
// pt_ref below); the back-pointer half of every pair is implied.
#pragma once
#include <cstdint>
#include <cfloat>
#include <climits>

#define TOPO_QUAL static __constant__ const
#include "topology_tables.inc"
#undef TOPO_QUAL

namespace dmtz {

typedef long long i64;

// Unsigned division by a divisor fixed for the whole grid, as a multiply-high
// and two shifts (Granlund and Montgomery, "Division by Invariant Integers
// using Multiplication", PLDI 1994, the N-bit round-up method of their
// Figure 4.1 with N = 64): with l = ceil(log2 d), m = floor(2^64 (2^l - d) / d)
// + 1, t = mulhi(m, n), q = (t + ((n - t) >> min(l, 1))) >> max(l - 1, 0) for
// every 64-bit n.  The id decodes below divide by grid extents; a 64-bit
// hardware division is a long instruction sequence on the GPU.
struct FDiv {
    unsigned long long d, m;
    int s1, s2;
};
static inline FDiv make_fdiv(unsigned long long d) {
    int l = 0;
    while (l < 64 && (1ull << l) < d) l++;
    const unsigned __int128 num = ((unsigned __int128)1 << 64) * (((unsigned __int128)1 << l) - d);
    FDiv f;
    f.d = d;
    f.m = (unsigned long long)(num / d) + 1;
    f.s1 = l < 1 ? l : 1;
    f.s2 = l > 1 ? l - 1 : 0;
    return f;
}
__host__ __device__ __forceinline__ unsigned long long fdiv(const FDiv &f, unsigned long long n) {
#ifdef __CUDA_ARCH__
    const unsigned long long t = __umul64hi(f.m, n);
#else
    const unsigned long long t = (unsigned long long)(((unsigned __int128)f.m * n) >> 64);
#endif
    return (t + ((n - t) >> f.s1)) >> f.s2;
}

struct Grid {
    int W, H, D;
    i64 WH, V, E, F, T;
    i64 eoff[8];   // first id of each edge family (eoff[7] = E)
    i64 bxy, byz, bxz;  // first ids of yz-plane, xz-plane, interior triangles
    i64 doff[14];  // linear offset of each stencil direction
    i64 coff[8];   // linear offset of each cube corner
    // 32-bit copies for grids of fewer than 2^31 vertices (small != 0): the
    // interior fast path indexes with 32-bit integers there
    int small;
    int WHi;
    int doff32[14];
    int coff32[8];
    // divisors of the id decodes: W, H, W-1, H-1, D-1, and the plane sizes
    // (W-1)H, W(H-1), W(D-1), (H-1)(D-1), (W-1)(D-1), (W-1)(H-1)
    FDiv dW, dH, dW1, dH1, dD1, dW1H, dWH1, dWD1, dH1D1, dW1D1, dW1H1;
};

static inline Grid make_grid(int W, int H, int D) {
    Grid g;
    g.W = W; g.H = H; g.D = D;
    const i64 w = W, h = H, d = D;
    g.WH = w * h;
    g.V = w * h * d;
    i64 c[7] = {(w - 1) * h * d, w * (h - 1) * d, w * h * (d - 1), (w - 1) * (h - 1) * d,
                w * (h - 1) * (d - 1), (w - 1) * h * (d - 1), (w - 1) * (h - 1) * (d - 1)};
    g.eoff[0] = 0;
    for (int k = 0; k < 7; k++) g.eoff[k + 1] = g.eoff[k] + c[k];
    g.E = g.eoff[7];
    g.bxy = 2 * d * (w - 1) * (h - 1);
    g.byz = g.bxy + 2 * w * (h - 1) * (d - 1);
    g.bxz = g.byz + 2 * h * (w - 1) * (d - 1);
    g.F = g.bxz + 6 * (w - 1) * (h - 1) * (d - 1);
    g.T = 6 * (w - 1) * (h - 1) * (d - 1);
    static const int dirs[14][3] = {{1, 0, 0},  {-1, 0, 0}, {0, 1, 0},  {0, -1, 0}, {0, 0, 1},
                                    {0, 0, -1}, {-1, 1, 0}, {1, -1, 0}, {0, 1, 1},  {0, -1, -1},
                                    {-1, 0, 1}, {1, 0, -1}, {-1, 1, 1}, {1, -1, -1}};
    for (int i = 0; i < 14; i++) g.doff[i] = dirs[i][0] + dirs[i][1] * w + dirs[i][2] * w * h;
    for (int c8 = 0; c8 < 8; c8++) g.coff[c8] = (c8 & 1) + ((c8 >> 1) & 1) * w + ((c8 >> 2) & 1) * w * h;
    g.small = g.V < (1LL << 31) ? 1 : 0;
    g.WHi = g.small ? (int)g.WH : 0;
    for (int i = 0; i < 14; i++) g.doff32[i] = g.small ? (int)g.doff[i] : 0;
    for (int c8 = 0; c8 < 8; c8++) g.coff32[c8] = g.small ? (int)g.coff[c8] : 0;
    g.dW = make_fdiv(w); g.dH = make_fdiv(h); g.dW1 = make_fdiv(w - 1); g.dH1 = make_fdiv(h - 1);
    g.dD1 = make_fdiv(d - 1); g.dW1H = make_fdiv((w - 1) * h); g.dWH1 = make_fdiv(w * (h - 1));
    g.dWD1 = make_fdiv(w * (d - 1)); g.dH1D1 = make_fdiv((h - 1) * (d - 1)); g.dW1D1 = make_fdiv((w - 1) * (d - 1));
    g.dW1H1 = make_fdiv((w - 1) * (h - 1));
    return g;
}

// ---------------------------------------------------------------------------
// Order keys.  compare_vertices (main_3d.cu:1043-1049) orders vertices by
// (value, id).  GB300 has a small float64 rate, so values are compared as
// order-preserving 64-bit integers: equal doubles (including -0 == +0) map to
// equal keys and the integer order equals the IEEE order for non-NaN input.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ uint64_t okey(double v) {
#ifdef __CUDA_ARCH__
    uint64_t b = (uint64_t)__double_as_longlong(v);
#else
    uint64_t b;
    __builtin_memcpy(&b, &v, 8);
#endif
    if (b == 0x8000000000000000ull) b = 0;
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
#define DMTZ_KEY_DBL_MAX 0xFFEFFFFFFFFFFFFFull  // okey(DBL_MAX)

__device__ __forceinline__ void decode_v(const Grid &g, i64 v, int &x, int &y, int &z) {
    const unsigned long long u = (unsigned long long)v, r = fdiv(g.dW, u), q = fdiv(g.dH, r);
    x = (int)(u - r * g.dW.d);
    y = (int)(r - q * g.dH.d);
    z = (int)q;
}
// n = (hi * B + mid) * C + lo with 0 <= mid < B, 0 <= lo < C, by the plane
// size BC and the row size C
__device__ __forceinline__ void split3(unsigned long long n, const FDiv &bc, const FDiv &c, int &hi, int &mid,
                                       int &lo) {
    const unsigned long long h = fdiv(bc, n), r = n - h * bc.d, m = fdiv(c, r);
    hi = (int)h;
    mid = (int)m;
    lo = (int)(r - m * c.d);
}
__device__ __forceinline__ bool inb(const Grid &g, int x, int y, int z) {
    return x >= 0 && x < g.W && y >= 0 && y < g.H && z >= 0 && z < g.D;
}
// cell with corners up to (mx,my,mz) exists at anchor (x,y,z)
__device__ __forceinline__ bool cell_ok(const Grid &g, int x, int y, int z, int mx, int my, int mz) {
    return x >= 0 && y >= 0 && z >= 0 && x + mx < g.W && y + my < g.H && z + mz < g.D;
}
__device__ __forceinline__ void corner_xyz(int c, int &dx, int &dy, int &dz) {
    dx = c & 1; dy = (c >> 1) & 1; dz = (c >> 2) & 1;
}
__device__ __forceinline__ int dir_of(int dx, int dy, int dz) {
    if (dx < -1 || dx > 1 || dy < -1 || dy > 1 || dz < -1 || dz > 1) return -1;
    return TOPO_DIR_LUT[(dx + 1) + 3 * (dy + 1) + 9 * (dz + 1)];
}
// maximum corner offsets of each cell kind (validity test)
__device__ __forceinline__ void edge_extent(int k, int &mx, int &my, int &mz) {
    int a = TOPO_EDGE_V[k][0] | TOPO_EDGE_V[k][1];
    corner_xyz(a, mx, my, mz);
}
__device__ __forceinline__ void face_extent(int s, int &mx, int &my, int &mz) {
    int a = TOPO_FACE_V[s][0] | TOPO_FACE_V[s][1] | TOPO_FACE_V[s][2];
    corner_xyz(a, mx, my, mz);
}

// ---------------------------------------------------------------------------
// Reference cell numbering (getEdgeID :917-1012, getTriangleID :246-423,
// getTetrahedraID :572-670) from (anchor, family/slot), and back.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ i64 edge_ref(const Grid &g, i64 x, i64 y, i64 z, int k) {
    const i64 W = g.W, H = g.H, D = g.D;
    switch (k) {
    case 0: return z * (W - 1) * H + y * (W - 1) + x;
    case 1: return g.eoff[1] + z * W * (H - 1) + x * (H - 1) + y;
    case 2: return g.eoff[2] + y * W * (D - 1) + x * (D - 1) + z;
    case 3: return g.eoff[3] + z * (H - 1) * (W - 1) + y * (W - 1) + x;
    case 4: return g.eoff[4] + x * (H - 1) * (D - 1) + y * (D - 1) + z;
    case 5: return g.eoff[5] + y * (W - 1) * (D - 1) + z * (W - 1) + x;
    default: return g.eoff[6] + z * (W - 1) * (H - 1) + y * (W - 1) + x;
    }
}
__host__ __device__ __forceinline__ i64 face_ref(const Grid &g, i64 x, i64 y, i64 z, int s) {
    const i64 W = g.W, H = g.H, D = g.D;
    if (s < 2) return 2 * (z * (W - 1) * (H - 1) + y * (W - 1) + x) + s;
    if (s < 4) return g.bxy + 2 * (x * (H - 1) * (D - 1) + y * (D - 1) + z) + (s - 2);
    if (s < 6) return g.byz + 2 * (y * (W - 1) * (D - 1) + z * (W - 1) + x) + (s - 4);
    return g.bxz + 6 * (z * (W - 1) * (H - 1) + y * (W - 1) + x) + (s - 6);
}
__host__ __device__ __forceinline__ i64 tet_ref(const Grid &g, i64 x, i64 y, i64 z, int s) {
    const i64 W = g.W, H = g.H;
    return 6 * (z * (W - 1) * (H - 1) + y * (W - 1) + x) + s;
}
// valid edge id -> anchor + family
__device__ __forceinline__ void edge_unref(const Grid &g, i64 e, int &x, int &y, int &z, int &k) {
    k = 0;
    while (k < 6 && e >= g.eoff[k + 1]) k++;
    const unsigned long long r = (unsigned long long)(e - g.eoff[k]);
    switch (k) {
    case 0: split3(r, g.dW1H, g.dW1, z, y, x); break;
    case 1: split3(r, g.dWH1, g.dH1, z, x, y); break;
    case 2: split3(r, g.dWD1, g.dD1, y, x, z); break;
    case 4: split3(r, g.dH1D1, g.dD1, x, y, z); break;
    case 5: split3(r, g.dW1D1, g.dW1, y, z, x); break;
    default: split3(r, g.dW1H1, g.dW1, z, y, x); break;
    }
}
__device__ __forceinline__ void face_unref(const Grid &g, i64 t, int &x, int &y, int &z, int &s) {
    if (t < g.bxy) {
        const unsigned long long u = (unsigned long long)t;
        s = (int)(u & 1);
        split3(u >> 1, g.dW1H1, g.dW1, z, y, x);
    } else if (t < g.byz) {
        const unsigned long long r = (unsigned long long)(t - g.bxy);
        s = 2 + (int)(r & 1);
        split3(r >> 1, g.dH1D1, g.dD1, x, y, z);
    } else if (t < g.bxz) {
        const unsigned long long r = (unsigned long long)(t - g.byz);
        s = 4 + (int)(r & 1);
        split3(r >> 1, g.dW1D1, g.dW1, y, z, x);
    } else {
        const unsigned long long r = (unsigned long long)(t - g.bxz), b = r / 6;
        s = 6 + (int)(r - 6 * b);
        split3(b, g.dW1H1, g.dW1, z, y, x);
    }
}
__device__ __forceinline__ void tet_unref(const Grid &g, i64 t, int &x, int &y, int &z, int &s) {
    const unsigned long long u = (unsigned long long)t, b = u / 6;
    s = (int)(u - 6 * b);
    split3(b, g.dW1H1, g.dW1, z, y, x);
}

// packed field accessors
// A slot in a list whose length is *n: the converged lanes appending to the
// same counter take one atomic between them (the leader's), so that a list
// filled from every warp does not serialise on one address.
__device__ __forceinline__ unsigned long long agg_slot(unsigned long long *n) {
    const unsigned act = __activemask();
    const unsigned peers = __match_any_sync(act, (unsigned long long)(uintptr_t)n);
    const int leader = __ffs(peers) - 1;
    const unsigned lane = threadIdx.x & 31u;
    unsigned long long base = 0;
    if ((int)lane == leader) base = atomicAdd(n, (unsigned long long)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    return base + (unsigned long long)__popc(peers & ((1u << lane) - 1u));
}
__device__ __forceinline__ int eup_get(uint32_t w, int k) { return (w >> (3 * k)) & 7; }
__device__ __forceinline__ int fup_get(uint32_t w, int s) { return (w >> (2 * s)) & 3; }

// Per-field device state (structure of arrays, one entry per anchor vertex)
struct FieldState {
    const double *val;   // field values (f or g)
    uint64_t *key;       // okey(val)
    uint16_t *low;       // bit i: neighbour i exists and is below this vertex
    uint8_t *pv;
    uint32_t *ea2;       // edge pass a2=0 result
    uint16_t *fp3;       // triangles paired after the first triangle pass
    uint32_t *fa3;       // triangle pass a2=0 result
    uint32_t *eup;       // final edge -> triangle
    uint32_t *fup;       // final triangle -> tetrahedron
    uint32_t *crit;      // bit 0 vertex, 1..7 edges, 8..19 triangles, 20..25 tetrahedra
    uint32_t *tcode;     // 6 x 3 bits: which facet (TOPO_TET_FACE order) each tetrahedron
                         // is paired with, 7 = unpaired or absent (may be null)
};

}  // namespace dmtz
