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
    x = (int)(v % g.W);
    i64 r = v / g.W;
    y = (int)(r % g.H);
    z = (int)(r / g.H);
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
    const i64 W = g.W, H = g.H, D = g.D;
    k = 0;
    while (k < 6 && e >= g.eoff[k + 1]) k++;
    i64 r = e - g.eoff[k];
    switch (k) {
    case 0: z = (int)(r / ((W - 1) * H)); y = (int)((r % ((W - 1) * H)) / (W - 1)); x = (int)(r % (W - 1)); break;
    case 1: z = (int)(r / (W * (H - 1))); x = (int)((r % (W * (H - 1))) / (H - 1)); y = (int)(r % (H - 1)); break;
    case 2: y = (int)(r / (W * (D - 1))); x = (int)((r % (W * (D - 1))) / (D - 1)); z = (int)(r % (D - 1)); break;
    case 4: x = (int)(r / ((H - 1) * (D - 1))); y = (int)((r % ((H - 1) * (D - 1))) / (D - 1)); z = (int)(r % (D - 1)); break;
    case 5: y = (int)(r / ((W - 1) * (D - 1))); z = (int)((r % ((W - 1) * (D - 1))) / (W - 1)); x = (int)(r % (W - 1)); break;
    default: z = (int)(r / ((W - 1) * (H - 1))); y = (int)((r % ((W - 1) * (H - 1))) / (W - 1)); x = (int)(r % (W - 1)); break;
    }
}
__device__ __forceinline__ void face_unref(const Grid &g, i64 t, int &x, int &y, int &z, int &s) {
    const i64 W = g.W, H = g.H, D = g.D;
    if (t < g.bxy) {
        i64 b = t / 2; s = (int)(t % 2);
        z = (int)(b / ((W - 1) * (H - 1))); y = (int)((b % ((W - 1) * (H - 1))) / (W - 1)); x = (int)(b % (W - 1));
    } else if (t < g.byz) {
        i64 r = t - g.bxy, b = r / 2; s = 2 + (int)(r % 2);
        x = (int)(b / ((H - 1) * (D - 1))); y = (int)((b % ((H - 1) * (D - 1))) / (D - 1)); z = (int)(b % (D - 1));
    } else if (t < g.bxz) {
        i64 r = t - g.byz, b = r / 2; s = 4 + (int)(r % 2);
        y = (int)(b / ((W - 1) * (D - 1))); z = (int)((b % ((W - 1) * (D - 1))) / (W - 1)); x = (int)(b % (W - 1));
    } else {
        i64 r = t - g.bxz, b = r / 6; s = 6 + (int)(r % 6);
        z = (int)(b / ((W - 1) * (H - 1))); y = (int)((b % ((W - 1) * (H - 1))) / (W - 1)); x = (int)(b % (W - 1));
    }
}
__device__ __forceinline__ void tet_unref(const Grid &g, i64 t, int &x, int &y, int &z, int &s) {
    const i64 W = g.W, H = g.H;
    i64 b = t / 6; s = (int)(t % 6);
    z = (int)(b / ((W - 1) * (H - 1))); y = (int)((b % ((W - 1) * (H - 1))) / (W - 1)); x = (int)(b % (W - 1));
}

// packed field accessors
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
