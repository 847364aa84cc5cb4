// dmtz.cu — kernels and host driver of libdmtz (see include/dmtz.h).
//
// Data layout in HBM, per field (original f, decompressed g), one entry per
// anchor vertex, structure of arrays:
//   key u64 | low u16 | pv u8 | ea2 u32 | fp3 u16 | fa3 u32 | eup u32 | fup u32 | crit u32
// plus, shared: f, g (float64), delta_counter (int32), request bits (1 bit per
// vertex), the request list and the four mismatch lists (cell ids, int64).
//
// One correction round (main_3d.cu:6789-6921) is: fix rules on the mismatch
// lists -> request bits/list; apply (bounded update of g); five pairing passes
// on g; criticality + mismatch compaction.  Counters live on the device; the
// host reads four words per round (or none, in the CUDA-graph loop).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <atomic>
#include <mutex>
#include <thread>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/dmtz.h"
#include "cnn.cuh"
#include "dmtz_common.cuh"
#include "pairing.cuh"
#include "pairing_fast.cuh"
#include "rules.cuh"

using namespace dmtz;

namespace dmtz {

static const int kBlock = 256;
static inline unsigned grid_for(i64 n) { return (unsigned)std::max<i64>(1, (n + kBlock - 1) / kBlock); }

// --------------------------------------------------------------- mismatch compaction
struct Lists {
    i64 *l[4];                  // min, 1-saddle, 2-saddle, max (reference cell ids)
    unsigned long long *n;      // 4 counters
    i64 cap[4];                 // capacities; a counter above its capacity = overflow,
                                // the host grows the list and scans again
};

__device__ __forceinline__ void push_list(const Lists &L, int k, i64 id) {
    const unsigned long long at = agg_slot(&L.n[k]);
    if ((i64)at < L.cap[k]) L.l[k][at] = id;
}

// mismatch between the decompressed and the original critical cells
// (get_false_minimum / saddle / 2_saddle / maximum, main_3d.cu:2492-2550):
// a scan of the two criticality masks, compacting mismatched cells' ids
__global__ void k_mismatch_scan(Grid g, const uint32_t *crit_d, const uint32_t *crit_o, Lists L, int want_saddles) {
    for (i64 v = (i64)blockIdx.x * blockDim.x + threadIdx.x; v < g.V; v += (i64)gridDim.x * blockDim.x) {
        uint32_t d = crit_d[v] ^ crit_o[v];
        if (!want_saddles) d &= 1u | (0x3Fu << 20);
        if (!d) continue;
        int x, y, z;
        decode_v(g, v, x, y, z);
        while (d) {
            const int b = __ffs(d) - 1;
            d &= d - 1;
            if (b == 0) push_list(L, 0, v);
            else if (b < 8) push_list(L, 1, edge_ref(g, x, y, z, b - 1));
            else if (b < 20) push_list(L, 2, face_ref(g, x, y, z, b - 8));
            else push_list(L, 3, tet_ref(g, x, y, z, b - 20));
        }
    }
}

// Incremental mismatch lists.  A cell's mismatch status changes only where
// its anchor's criticality mask was recomputed, i.e. in the bricks of the
// round's criticality pass (marked fresh).  The new lists are the old entries
// outside fresh bricks plus a scan of the fresh bricks' anchors, built in T
// and copied back.  Valid when every scan of the run uses the same saddle
// flag and the old lists were complete (an overflow is followed by a full
// scan before the next round).
__global__ void k_mark_fresh(const uint32_t *list, const unsigned long long *n, uint8_t *fresh, int nbx, int nby) {
    const i64 nb = (i64)*n;
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += (i64)gridDim.x * blockDim.x) {
        const uint32_t e = list[i];
        fresh[(e & 0x7FF) + (i64)nbx * (((e >> 11) & 0x7FF) + (i64)nby * (e >> 22))] = 1;
    }
}
__global__ void k_list_keep(Grid g, Lists L, Lists T, const uint8_t *fresh, int sx, int sy, int sz, int nbx, int nby) {
    const i64 n0 = min((i64)L.n[0], L.cap[0]), n1 = min((i64)L.n[1], L.cap[1]), n2 = min((i64)L.n[2], L.cap[2]),
              n3 = min((i64)L.n[3], L.cap[3]);
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n0 + n1 + n2 + n3; i += (i64)gridDim.x * blockDim.x) {
        int k, x, y, z, sl;
        i64 id;
        if (i < n0) {
            k = 0;
            id = L.l[0][i];
            decode_v(g, id, x, y, z);
        } else if (i < n0 + n1) {
            k = 1;
            id = L.l[1][i - n0];
            edge_unref(g, id, x, y, z, sl);
        } else if (i < n0 + n1 + n2) {
            k = 2;
            id = L.l[2][i - n0 - n1];
            face_unref(g, id, x, y, z, sl);
        } else {
            k = 3;
            id = L.l[3][i - n0 - n1 - n2];
            tet_unref(g, id, x, y, z, sl);
        }
        if (fresh[x / sx + (i64)nbx * (y / sy + (i64)nby * (z / sz))]) continue;
        push_list(T, k, id);
    }
}
// the anchors of the fresh bricks (one block per listed brick step)
__global__ void k_scan_fresh(Grid g, const uint32_t *crit_d, const uint32_t *crit_o, Lists T, const uint32_t *blist,
                             const unsigned long long *bn, int sx, int sy, int sz, int want_saddles) {
    const i64 nb = (i64)*bn;
    const int per = sx * sy * sz;
    for (i64 b = blockIdx.x; b < nb; b += gridDim.x) {
        const uint32_t e = blist[b];
        const int x0 = (e & 0x7FF) * sx, y0 = ((e >> 11) & 0x7FF) * sy, z0 = (e >> 22) * sz;
        for (int t = threadIdx.x; t < per; t += blockDim.x) {
            const int x = x0 + t % sx, y = y0 + (t / sx) % sy, z = z0 + t / (sx * sy);
            if (x >= g.W || y >= g.H || z >= g.D) continue;
            const i64 v = x + (i64)y * g.W + (i64)z * g.WH;
            uint32_t d = crit_d[v] ^ crit_o[v];
            if (!want_saddles) d &= 1u | (0x3Fu << 20);
            while (d) {
                const int bit = __ffs(d) - 1;
                d &= d - 1;
                if (bit == 0) push_list(T, 0, v);
                else if (bit < 8) push_list(T, 1, edge_ref(g, x, y, z, bit - 1));
                else if (bit < 20) push_list(T, 2, face_ref(g, x, y, z, bit - 8));
                else push_list(T, 3, tet_ref(g, x, y, z, bit - 20));
            }
        }
    }
}
// T back into L (counts included; entries past a list's capacity were not
// stored, and the count shows the overflow)
__global__ void k_list_back(Lists T, Lists L) {
    const i64 n0 = min((i64)T.n[0], T.cap[0]), n1 = min((i64)T.n[1], T.cap[1]), n2 = min((i64)T.n[2], T.cap[2]),
              n3 = min((i64)T.n[3], T.cap[3]);
    const i64 tid = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    for (i64 i = tid; i < n0 + n1 + n2 + n3; i += (i64)gridDim.x * blockDim.x) {
        if (i < n0) L.l[0][i] = T.l[0][i];
        else if (i < n0 + n1) L.l[1][i - n0] = T.l[1][i - n0];
        else if (i < n0 + n1 + n2) L.l[2][i - n0 - n1] = T.l[2][i - n0 - n1];
        else L.l[3][i - n0 - n1 - n2] = T.l[3][i - n0 - n1 - n2];
    }
    if (tid < 4) L.n[tid] = T.n[tid];
}

// Dirty bricks, per pass.  The gradient state of an anchor depends on values
// at most r_p anchors away in pass p: r = 1 (vertex pass), 2 (edge pass),
// 3 (first triangle pass, -3..2), 3 (second edge pass), 4 (second triangle
// pass), 5 (criticality, -5..4).  For every changed vertex, each brick within
// 5 anchors gets bit r-1 for every r >= its distance (the largest per-axis gap
// between the vertex and the brick's anchors); pass p re-pairs the bricks with
// bit r_p - 1.  Flags are bytes packed four to a word (atomicOr on the word).
constexpr int kRadii = 5;
__global__ void k_mark_dirty(Grid g, int nbx, int nby, int nbz, int sx, int sy, int sz, const i64 *verts,
                             const unsigned long long *nverts, uint32_t *flags) {
    const i64 n = (i64)*nverts;
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        int x, y, z;
        decode_v(g, verts[i], x, y, z);
        const int x0 = max(x - kRadii, 0) / sx, x1 = min(x + kRadii, g.W - 1) / sx;
        const int y0 = max(y - kRadii, 0) / sy, y1 = min(y + kRadii, g.H - 1) / sy;
        const int z0 = max(z - kRadii, 0) / sz, z1 = min(z + kRadii, g.D - 1) / sz;
        for (int bz = z0; bz <= z1; bz++) {
            const int dz = max(0, max(bz * sz - z, z - (bz * sz + sz - 1)));
            for (int by = y0; by <= y1; by++) {
                const int dy = max(0, max(by * sy - y, y - (by * sy + sy - 1)));
                for (int bx = x0; bx <= x1; bx++) {
                    const int dx = max(0, max(bx * sx - x, x - (bx * sx + sx - 1)));
                    const int d = max(dx, max(dy, dz));  // <= kRadii by the loop bounds
                    const uint32_t mask = 0x1Fu & ~((1u << max(d - 1, 0)) - 1u);
                    const i64 b = bx + (i64)nbx * (by + (i64)nby * bz);
                    atomicOr(&flags[b >> 2], mask << (8 * (b & 3)));
                }
            }
        }
    }
}
// Walk-cache tiles: 16^3 anchors.  Every brick the criticality pass re-pairs
// marks the tiles it overlaps (a brick spans at most 3 tiles per axis).
constexpr int kTile = 16, kTileShift = 4;
__global__ void k_mark_tiles(const uint32_t *list, const unsigned long long *n, int sx, int sy, int sz, int ntx,
                             int nty, int ntz, uint8_t *dirty) {
    const i64 nb = (i64)*n;
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += (i64)gridDim.x * blockDim.x) {
        const uint32_t e = list[i];
        const int bx = e & 0x7FF, by = (e >> 11) & 0x7FF, bz = e >> 22;
        const int x0 = (bx * sx) >> kTileShift, x1 = min((bx * sx + sx - 1) >> kTileShift, ntx - 1);
        const int y0 = (by * sy) >> kTileShift, y1 = min((by * sy + sy - 1) >> kTileShift, nty - 1);
        const int z0 = (bz * sz) >> kTileShift, z1 = min((bz * sz + sz - 1) >> kTileShift, ntz - 1);
        for (int tz = z0; tz <= z1; tz++)
            for (int ty = y0; ty <= y1; ty++)
                for (int tx = x0; tx <= x1; tx++) dirty[tx + (i64)ntx * (ty + (i64)nty * tz)] = 1;
    }
}
// one compacted brick list per radius (list r-1 holds the bricks with bit
// r-1), and the flags cleared for the next round
__global__ void k_compact_bricks(int nbx, int nby, int nbz, uint32_t *flags, uint32_t *lists, i64 stride,
                                 unsigned long long *n) {
    const i64 nb = (i64)nbx * nby * nbz;
    for (i64 w = (i64)blockIdx.x * blockDim.x + threadIdx.x; w < (nb + 3) / 4; w += (i64)gridDim.x * blockDim.x) {
        const uint32_t word = flags[w];
        if (!word) continue;
        flags[w] = 0;
        for (int q = 0; q < 4; q++) {
            const uint32_t m = (word >> (8 * q)) & 0xFFu;
            if (!m) continue;
            const i64 b = 4 * w + q;
            const int bx = (int)(b % nbx), by = (int)((b / nbx) % nby), bz = (int)(b / ((i64)nbx * nby));
            const uint32_t code = (uint32_t)bx | ((uint32_t)by << 11) | ((uint32_t)bz << 22);
            for (int r = 0; r < kRadii; r++)
                if (m & (1u << r)) lists[r * stride + (i64)atomicAdd(&n[r], 1ull)] = code;
        }
    }
}

// --------------------------------------------------------------- export to the reference layout
__global__ void k_export(Grid g, FieldState s, int32_t *PV, int32_t *PE, int32_t *PF, int32_t *PT) {
    i64 v = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= g.V) return;
    int x, y, z;
    decode_v(g, v, x, y, z);
    const int d = s.pv[v];
    PV[v] = d == 15 ? -1 : (int32_t)edge_ref_pair(g, v, v + g.doff[d]);
    const uint32_t eu = s.eup[v];
    for (int k = 0; k < 7; k++) {
        int mx, my, mz;
        edge_extent(k, mx, my, mz);
        if (!cell_ok(g, x, y, z, mx, my, mz)) continue;
        i64 val = -1;
        const int up = eup_get(eu, k);
        if (up) {
            const signed char *cf = TOPO_EDGE_COF[k][up - 1];
            val = face_ref(g, x + cf[0], y + cf[1], z + cf[2], cf[3]);
        } else {
            const int cp = TOPO_EDGE_V[k][0], cq = TOPO_EDGE_V[k][1];
            const i64 p = v + g.coff[cp], q = v + g.coff[cq];
            if (s.pv[p] == TOPO_CORNER_DIR[cp][cq]) val = p;
            else if (s.pv[q] == TOPO_CORNER_DIR[cq][cp]) val = q;
        }
        PE[edge_ref(g, x, y, z, k)] = (int32_t)val;
    }
    const uint32_t fu = s.fup[v];
    for (int sl = 0; sl < 12; sl++) {
        int mx, my, mz;
        face_extent(sl, mx, my, mz);
        if (!cell_ok(g, x, y, z, mx, my, mz)) continue;
        i64 val = -1;
        const int up = fup_get(fu, sl);
        if (up) {
            const signed char *tc = TOPO_FACE_COF[sl][up - 1];
            val = tet_ref(g, x + tc[0], y + tc[1], z + tc[2], tc[3]);
        } else {
            for (int j = 0; j < 3; j++) {
                const signed char *fe = TOPO_FACE_EDGE[sl][j];
                const i64 ea = v + fe[0] + (i64)fe[1] * g.W + (i64)fe[2] * g.WH;
                if (eup_get(s.eup[ea], fe[3]) == fe[4] + 1) val = edge_ref(g, x + fe[0], y + fe[1], z + fe[2], fe[3]);
            }
        }
        PF[face_ref(g, x, y, z, sl)] = (int32_t)val;
    }
    if (cell_ok(g, x, y, z, 1, 1, 1)) {
        for (int ts = 0; ts < 6; ts++) {
            i64 val = -1;
            for (int j = 0; j < 4; j++) {
                const signed char *tf = TOPO_TET_FACE[ts][j];
                const i64 fa = v + tf[0] + (i64)tf[1] * g.W + (i64)tf[2] * g.WH;
                if (fup_get(s.fup[fa], tf[3]) == tf[4] + 1) val = face_ref(g, x + tf[0], y + tf[1], z + tf[2], tf[3]);
            }
            PT[tet_ref(g, x, y, z, ts)] = (int32_t)val;
        }
    }
}

// --------------------------------------------------------------- fix rules
struct CpLists {
    const i64 *l[4];
    const unsigned long long *n;
    i64 cap[4];
};

// fix_minimum, [fix_saddle, fix_2saddle], fix_maximum over the current lists
// (the host never runs this on an overflowed list; the clamp only keeps
// every read inside the allocation).  Two forms, chosen on the device from
// the list lengths, so that a graph can hold both: when every listed cell
// fits one pass of the grid (`pass` threads), k_fix_cp gives each thread one
// cell of the concatenated lists and the four rules' latency chains overlap;
// longer lists (the first rounds of noisy fields: millions of cells) go to
// one kernel per cell type, k_fix_cp_t, whose code holds one rule tree: in one
// kernel the four case trees thrashed the instruction cache (a few active
// lanes per warp, warps stalled on instruction fetch).  The rules only set
// request bits, so neither form changes the result.
__device__ __forceinline__ void cp_counts(const CpLists &L, int preserve_saddles, i64 n[4]) {
    n[0] = min((i64)L.n[0], L.cap[0]);
    n[1] = preserve_saddles ? min((i64)L.n[1], L.cap[1]) : 0;
    n[2] = preserve_saddles ? min((i64)L.n[2], L.cap[2]) : 0;
    n[3] = min((i64)L.n[3], L.cap[3]);
}
__global__ void k_fix_cp(RuleCtx c, CpLists L, int preserve_saddles, i64 pass) {
    i64 n[4];
    cp_counts(L, preserve_saddles, n);
    if (n[0] + n[1] + n[2] + n[3] > pass) return;  // the per-type kernels take it
    i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n[0]) { rule_min(c, L.l[0][i]); return; }
    i -= n[0];
    if (i < n[1]) { rule_saddle(c, L.l[1][i]); return; }
    i -= n[1];
    if (i < n[2]) { rule_2saddle(c, L.l[2][i]); return; }
    i -= n[2];
    if (i < n[3]) rule_max(c, L.l[3][i]);
}
template <int T>
__global__ void k_fix_cp_t(RuleCtx c, CpLists L, int preserve_saddles, i64 pass) {
    i64 n[4];
    cp_counts(L, preserve_saddles, n);
    if (n[0] + n[1] + n[2] + n[3] <= pass) return;  // k_fix_cp took it
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n[T]; i += (i64)gridDim.x * blockDim.x) {
        if (T == 0) rule_min(c, L.l[0][i]);
        else if (T == 1) rule_saddle(c, L.l[1][i]);
        else if (T == 2) rule_2saddle(c, L.l[2][i]);
        else rule_max(c, L.l[3][i]);
    }
}
// the critical-point fix round; returns the number of kernels launched
inline int launch_fix_cp(const RuleCtx &rc, const CpLists &L, int ps, unsigned grid, cudaStream_t st) {
    const i64 pass = (i64)grid * kBlock;
    k_fix_cp<<<grid, kBlock, 0, st>>>(rc, L, ps, pass);
    k_fix_cp_t<0><<<grid, kBlock, 0, st>>>(rc, L, ps, pass);
    if (ps) {
        k_fix_cp_t<1><<<grid, kBlock, 0, st>>>(rc, L, ps, pass);
        k_fix_cp_t<2><<<grid, kBlock, 0, st>>>(rc, L, ps, pass);
    }
    k_fix_cp_t<3><<<grid, kBlock, 0, st>>>(rc, L, ps, pass);
    return ps ? 5 : 3;
}

// separatrix records
struct PathRec {
    i64 *as_tet, *as_cur, *ds_edge, *ds_vert;
    unsigned long long *n;  // [0] ascending, [1] descending
    i64 cap_as, cap_ds;     // at most one record per original 2-saddle / 1-saddle
};

// Original ascending paths (is_false, main_3d.cu:4437-4497) step from a
// tetrahedron through the facet it is paired with to that facet's other
// coface (get_cell_tetra's other one; none = the path leaves the grid).  The
// original gradient is fixed during a correction, so each tetrahedron's
// successor is computed once and stored in one byte: the successor's anchor
// offset ((dx+1) + 3(dy+1) + 9(dz+1), each in -1..1) times 6 plus its slot;
// 255 = the path ends (a maximum, or a boundary facet).  The six bytes of an
// anchor's tetrahedra share one 8-byte word (one coalesced store).  The
// reference's back-pointer test on the way is always true for a consistent
// gradient.
__device__ __forceinline__ uint8_t asc_step(const Grid &g, int x, int y, int z, int ts, uint32_t tc) {
    const int j = (tc >> (3 * ts)) & 7;
    if (j == 7) return 255;
    const signed char *tf = TOPO_TET_FACE[ts][j];
    const int fs = tf[3], other = 1 - tf[4];
    if (other >= TOPO_FACE_NCOF[fs]) return 255;
    const signed char *oc = TOPO_FACE_COF[fs][other];
    const int dx = tf[0] + oc[0], dy = tf[1] + oc[1], dz = tf[2] + oc[2];
    if (!cell_ok(g, x + dx, y + dy, z + dz, 1, 1, 1)) return 255;
    return (uint8_t)(((dx + 1) + 3 * (dy + 1) + 9 * (dz + 1)) * 6 + oc[3]);
}
// asc_step with the tetrahedron slot TS fixed at compile time: the facet and
// coface tables become immediates (runtime-indexed table reads with different
// indices across a warp are served one index at a time)
template <int TS>
__device__ __forceinline__ uint8_t asc_step_c(const Grid &g, int x, int y, int z, uint32_t tc) {
    const int j = (tc >> (3 * TS)) & 7;
    uint8_t out = 255;
    DMTZ_FOR(4, J, {
        constexpr int jj = decltype(J)::value;
        constexpr int fs = cxt::TOPO_TET_FACE[TS][jj][3], other = 1 - cxt::TOPO_TET_FACE[TS][jj][4];
        if constexpr (other < cxt::TOPO_FACE_NCOF[fs]) {
            constexpr int dx = cxt::TOPO_TET_FACE[TS][jj][0] + cxt::TOPO_FACE_COF[fs][other][0],
                          dy = cxt::TOPO_TET_FACE[TS][jj][1] + cxt::TOPO_FACE_COF[fs][other][1],
                          dz = cxt::TOPO_TET_FACE[TS][jj][2] + cxt::TOPO_FACE_COF[fs][other][2],
                          os = cxt::TOPO_FACE_COF[fs][other][3];
            constexpr uint8_t code = (uint8_t)(((dx + 1) + 3 * (dy + 1) + 9 * (dz + 1)) * 6 + os);
            if (j == jj) out = cell_ok(g, x + dx, y + dy, z + dz, 1, 1, 1) ? code : (uint8_t)255;
        }
    });
    return out;
}
__global__ void k_path_succ(Grid g, const uint32_t *tcodeP, uint8_t *succ) {
    i64 v = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= g.V) return;
    int x, y, z;
    decode_v(g, v, x, y, z);
    const bool cube = cell_ok(g, x, y, z, 1, 1, 1);
    const uint32_t tc = tcodeP[v];
    uint64_t packed = 0xFFFF000000000000ull;
    DMTZ_FOR(6, TS, {
        constexpr int ts = decltype(TS)::value;
        const uint8_t out = cube ? asc_step_c<ts>(g, x, y, z, tc) : (uint8_t)255;
        packed |= (uint64_t)out << (8 * ts);
    });
    reinterpret_cast<uint64_t *>(succ)[v] = packed;
}

// compact list of original critical cells of one dimension: criticality
// bits FIRST .. FIRST+SLOTS-1 of an anchor (SLOTS cells per anchor), entry =
// anchor * SLOTS + slot.  The 2-saddle triangles: <8, 12>; the 1-saddle
// edges: <1, 7>.
template <int FIRST, int SLOTS>
__global__ void k_crit_list(Grid g, const uint32_t *critP, i64 *list, i64 cap, unsigned long long *n) {
    // a block takes kBlock x 8 consecutive anchors per step: each thread
    // counts its 8 anchors' 2-saddles, a block scan places them in anchor
    // order, and one atomic per block step reserves the block's range (one
    // atomic per warp over the whole grid serialised this kernel on the
    // counter)
    __shared__ unsigned wtot[kBlock / 32];
    __shared__ unsigned long long bbase;
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5, full = 0xffffffffu;
    const i64 per = (i64)kBlock * 8;
    for (i64 b0 = (i64)blockIdx.x * per; b0 < g.V; b0 += (i64)gridDim.x * per) {
        const i64 v0 = b0 + (i64)threadIdx.x * 8;
        uint32_t m[8];
        unsigned mine = 0;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            m[j] = v0 + j < g.V ? (critP[v0 + j] >> FIRST) & ((1u << SLOTS) - 1u) : 0u;
            mine += __popc(m[j]);
        }
        unsigned incl = mine;
        for (int off = 1; off < 32; off <<= 1) {
            const unsigned y = __shfl_up_sync(full, incl, off);
            if (lane >= (unsigned)off) incl += y;
        }
        if (lane == 31) wtot[warp] = incl;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long t = 0;
            for (int w = 0; w < kBlock / 32; w++) {
                const unsigned c = wtot[w];
                wtot[w] = (unsigned)t;
                t += c;
            }
            bbase = t ? atomicAdd(n, t) : 0ull;
        }
        __syncthreads();
        unsigned long long at = bbase + wtot[warp] + incl - mine;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            uint32_t mm = m[j];
            while (mm) {
                const int sl = __ffs(mm) - 1;
                mm &= mm - 1;
                if ((i64)at < cap) list[at] = (v0 + j) * SLOTS + sl;
                at++;
            }
        }
        __syncthreads();  // wtot and bbase are reused by the next step
    }
}

// numbers of original 1-saddle edges (out[0]) and 2-saddle triangles (out[1])
__global__ void k_count_saddles(i64 V, const uint32_t *critP, unsigned long long *out) {
    unsigned long long a = 0, b = 0;
    for (i64 v = (i64)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (i64)gridDim.x * blockDim.x) {
        const uint32_t m = critP[v];
        a += __popc((m >> 1) & 0x7Fu);
        b += __popc((m >> 8) & 0xFFFu);
    }
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, off);
        b += __shfl_down_sync(0xffffffffu, b, off);
    }
    if ((threadIdx.x & 31) == 0) {
        if (a) atomicAdd(&out[0], a);
        if (b) atomicAdd(&out[1], b);
    }
}

// ------------------------------------------------------------------- walls
// preserve_connectors = 1: get_false_ds_wall (main_3d.cu:5064-5121) restated
// without its races.  Every original 2-saddle face runs its own depth-first
// search over the faces reachable by original V-paths, in the reference's
// order: pop a face; if it was not visited, take its edges (v1 v2), (v1 v3),
// (v2 v3) of its descending vertex triple; skip an originally critical edge;
// the first edge whose original and decompressed pairings differ is the
// record; otherwise push the face the edge is originally paired with (when
// it is a face and not this one).
//
// Visited marks are a direct-mapped cache of face ids.  A face found there was
// visited and is skipped; a visited face that fell out of the cache is
// searched again, which never changes the record: V-paths have no cycles and
// the stack finishes a face's descendants before the entries below it, so
// every face reachable from a visited face was visited before it comes back,
// and a repeat only re-checks edges that passed and pushes visited faces.  The
// cache size bounds only the work.  A search that passes its pop limit or
// outgrows its stack is handed to the next tier (larger stack, cache and pop
// limit in device scratch memory); the record does not depend on the tier.
struct WallRec {
    i64 *sad, *edge;        // record: 2-saddle face, first differing edge of its wall
    unsigned long long *n;
    i64 cap;
};
constexpr int kWallStack1 = 24, kWallCacheBits1 = 6;
constexpr long long kWallPops1 = 1024;

__device__ __forceinline__ unsigned wall_slot(i64 t, int bits) {
    return (unsigned)(((unsigned long long)t * 0x9E3779B97F4A7C15ull) >> (64 - bits));
}
// 0: no differing edge, 1: record in rec, 2: stack or pop limit reached
__device__ int wall_dfs(const RuleCtx &c, i64 sad, i64 *stack, int stack_cap, i64 *cache, int cache_bits,
                        long long pop_cap, i64 &rec) {
    const Grid &G = c.g;
    int top = 0;
    stack[top++] = sad;
    long long pops = 0;
    while (top > 0) {
        const i64 t = stack[--top];
        if (++pops > pop_cap) return 2;
        const unsigned slot = wall_slot(t, cache_bits);
        if (cache[slot] == t) continue;
        cache[slot] = t;
        i64 v1, v2, v3;
        tri_verts(G, t, v1, v2, v3);
        const i64 es[3] = {edge_ref_pair(G, v1, v2), edge_ref_pair(G, v1, v3), edge_ref_pair(G, v2, v3)};
        for (int k = 0; k < 3; k++) {
            const i64 j = es[k];
            const i64 pe = pe_ref(c, c.P, j);
            if (pe == -1) continue;
            if (pe != pe_ref(c, c.Q, j)) {
                rec = j;
                return 1;
            }
            if (pe != t && pe >= 0 && pe < G.F && pf_ref(c, c.P, pe) == j) {
                if (top == stack_cap) return 2;
                stack[top++] = pe;
            }
        }
    }
    return 0;
}
__device__ __forceinline__ void wall_emit(const WallRec &W, i64 s, i64 e) {
    const unsigned long long k = atomicAdd(W.n, 1ull);
    if ((i64)k < W.cap) {
        W.sad[k] = s;
        W.edge[k] = e;
    }
}
__device__ __forceinline__ void wall_defer(i64 *list, unsigned long long *n, i64 cap, i64 s) {
    const unsigned long long k = atomicAdd(n, 1ull);
    if ((i64)k < cap) list[k] = s;
}
// first tier: every original 2-saddle (sad2 codes anchor * 12 + slot), stack
// and cache in per-thread local memory
__global__ void k_wall_t1(RuleCtx c, const i64 *sad2, const unsigned long long *nsad, i64 capsad, WallRec W,
                          i64 *next, unsigned long long *nnext, i64 capnext) {
    const i64 n = min((i64)*nsad, capsad);
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        const i64 code = sad2[i];
        int x, y, z;
        decode_v(c.g, code / 12, x, y, z);
        const i64 sf = face_ref(c.g, x, y, z, (int)(code % 12));
        i64 stack[kWallStack1], cache[1 << kWallCacheBits1];
#pragma unroll
        for (int k = 0; k < (1 << kWallCacheBits1); k++) cache[k] = -1;
        i64 rec = -1;
        const int r = wall_dfs(c, sf, stack, kWallStack1, cache, kWallCacheBits1, kWallPops1, rec);
        if (r == 1) wall_emit(W, sf, rec);
        else if (r == 2) wall_defer(next, nnext, capnext, sf);
    }
}
// a larger tier for list[first, first + count): one thread per 2-saddle face,
// its stack and cache in scratch (stack_cap + 2^cache_bits entries each)
__global__ void k_wall_tn(RuleCtx c, const i64 *list, i64 first, i64 count, WallRec W, i64 *next,
                          unsigned long long *nnext, i64 capnext, i64 *scratch, int stack_cap, int cache_bits,
                          long long pop_cap) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (i64)gridDim.x * blockDim.x) {
        const i64 sf = list[first + i];
        i64 *stack = scratch + i * ((i64)stack_cap + ((i64)1 << cache_bits));
        i64 *cache = stack + stack_cap;
        for (i64 k = 0; k < ((i64)1 << cache_bits); k++) cache[k] = -1;
        i64 rec = -1;
        const int r = wall_dfs(c, sf, stack, stack_cap, cache, cache_bits, pop_cap, rec);
        if (r == 1) wall_emit(W, sf, rec);
        else if (r == 2) wall_defer(next, nnext, capnext, sf);
    }
}
__global__ void k_fix_wall(RuleCtx c, WallRec W) {
    const i64 n = min((i64)*W.n, W.cap);
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
        rule_ds_wall(c, W.edge[i]);
}

// ------------------------------------------------- connectivity-mode separatrices
// (preserve_vpath=1, preserve_geometry=0): a separatrix counts as false when
// its end differs, not its geometry.
//
// End of the descending path from vertex v under vertex directions pv: the
// minimum reached (the walks of get_orginal_saddle_min_pairs and
// get_false_ds_vpath_connectivity, main_3d.cu:4613-4687, 4961-5062).  With pvo
// given, trouble (if still -1) becomes the first vertex on the way whose
// direction under pvo differs (the reference's trouble_maker; it compares
// before stepping, never at the end vertex).
__device__ i64 desc_end(const Grid &g, const uint8_t *pv, const uint8_t *pvo, i64 v, i64 &trouble, i64 cap,
                        int *err) {
    for (i64 steps = 0;; steps++) {
        const int d = pv[v];
        if (d == 15) return v;
        if (pvo && trouble < 0 && pvo[v] != d) trouble = v;
        v += g.doff[d];
        if (steps > cap) {
            atomicOr(err, ERR_WALK);
            return v;
        }
    }
}
// End of the ascending path from tetrahedron (x, y, z, s) under tet codes tc:
// the maximum reached (reference id) or -1 when the path leaves the grid
// (get_paired_id, main_3d.cu:4499-4537)
__device__ i64 asc_end(const Grid &g, const uint32_t *tc, int x, int y, int z, int s, i64 cap, int *err) {
    for (i64 steps = 0;; steps++) {
        const uint32_t code = tc[x + (i64)y * g.W + (i64)z * g.WH];
        if (((code >> (3 * s)) & 7) == 7) return tet_ref(g, x, y, z, s);
        const int s8 = asc_step(g, x, y, z, s, code);
        if (s8 == 255) return -1;
        const int d = s8 / 6;
        s = s8 - 6 * d;
        x += d % 3 - 1;
        y += (d / 3) % 3 - 1;
        z += d / 9 - 1;
        if (steps > cap) {
            atomicOr(err, ERR_WALK);
            return -1;
        }
    }
}
// is_false (main_3d.cu:4437-4497): along the original ascending path from the
// tetrahedron, the first one whose decompressed pairing differs (into cur)
__device__ bool first_diff(const Grid &g, const uint32_t *tcP, const uint32_t *tcQ, const uint8_t *succ, int x, int y,
                           int z, int s, i64 cap, int *err, i64 &cur) {
    for (i64 steps = 0;; steps++) {
        const i64 ci = x + (i64)y * g.W + (i64)z * g.WH;
        const int p = (tcP[ci] >> (3 * s)) & 7;
        if (p == 7) return false;
        if (p != (int)((tcQ[ci] >> (3 * s)) & 7)) {
            cur = tet_ref(g, x, y, z, s);
            return true;
        }
        const int s8 = succ[ci * 8 + s];
        if (s8 == 255) return false;
        const int d = s8 / 6;
        s = s8 - 6 * d;
        x += d % 3 - 1;
        y += (d / 3) % 3 - 1;
        z += d / 9 - 1;
        if (steps > cap) {
            atomicOr(err, ERR_WALK);
            return false;
        }
    }
}
// get_false_ds_vpath_connectivity (main_3d.cu:4961-5062): for each original
// 1-saddle edge, the decompressed descending paths from its endpoints (v1,
// the higher id, first) against the original ones; the first endpoint whose
// minimum differs records (edge, trouble maker), the trouble maker carried
// over from v1's walk into v2's as in the reference.
__global__ void k_conn_ds(RuleCtx c, PathRec R, i64 cap) {
    const Grid &g = c.g;
    for (i64 v = (i64)blockIdx.x * blockDim.x + threadIdx.x; v < g.V; v += (i64)gridDim.x * blockDim.x) {
        uint32_t m = (c.P.crit[v] >> 1) & 0x7Fu;
        if (!m) continue;
        int x, y, z;
        decode_v(g, v, x, y, z);
        while (m) {
            const int k = __ffs(m) - 1;
            m &= m - 1;
            const i64 ends[2] = {v + g.coff[TOPO_EDGE_V[k][0]], v + g.coff[TOPO_EDGE_V[k][1]]};
            i64 trouble = -1, unused = -1;
            for (int j = 0; j < 2; j++) {
                const i64 eq = desc_end(g, c.Q.pv, c.P.pv, ends[j], trouble, cap, c.err);
                const i64 ep = desc_end(g, c.P.pv, nullptr, ends[j], unused, cap, c.err);
                if (eq != ep) {
                    const unsigned long long at = atomicAdd(&R.n[1], 1ull);
                    if ((i64)at < R.cap_ds) {
                        R.ds_edge[at] = edge_ref(g, x, y, z, k);
                        R.ds_vert[at] = trouble;
                    }
                    break;
                }
            }
        }
    }
}
// get_false_as_vpath_connectivity (main_3d.cu:4761-4835) as intended: for each
// decompressed 2-saddle triangle, its cofaces in search order; a coface whose
// decompressed ascending path ends at another maximum than the original one
// (the original end is -1 for triangles that are not original 2-saddles, the
// reference's initial value) is checked with is_false, and the first record
// ends the triangle.  The reference indexes its table of original ends by the
// direction loop's counter instead of the triangle (all triangles share 28
// slots, written concurrently), so its own result depends on scheduling.
__global__ void k_conn_as(Grid g, const uint32_t *critP, const uint32_t *critQ, const uint32_t *tcP,
                          const uint32_t *tcQ, const uint8_t *succ, PathRec R, i64 cap, int *err) {
    for (i64 v = (i64)blockIdx.x * blockDim.x + threadIdx.x; v < g.V; v += (i64)gridDim.x * blockDim.x) {
        uint32_t m = (critQ[v] >> 8) & 0xFFFu;
        if (!m) continue;
        const uint32_t mp = (critP[v] >> 8) & 0xFFFu;
        int x, y, z;
        decode_v(g, v, x, y, z);
        while (m) {
            const int sl = __ffs(m) - 1;
            m &= m - 1;
            for (int j = 0; j < TOPO_FACE_NCOF[sl]; j++) {
                const signed char *tc = TOPO_FACE_COF[sl][j];
                const int cx = x + tc[0], cy = y + tc[1], cz = z + tc[2], cs = tc[3];
                if (!cell_ok(g, cx, cy, cz, 1, 1, 1)) continue;
                const i64 eq = asc_end(g, tcQ, cx, cy, cz, cs, cap, err);
                const i64 ep = ((mp >> sl) & 1u) ? asc_end(g, tcP, cx, cy, cz, cs, cap, err) : -1;
                if (eq == ep) continue;
                i64 cur;
                if (first_diff(g, tcP, tcQ, succ, cx, cy, cz, cs, cap, err, cur)) {
                    const unsigned long long at = atomicAdd(&R.n[0], 1ull);
                    if ((i64)at < R.cap_as) {
                        R.as_tet[at] = tet_ref(g, cx, cy, cz, cs);
                        R.as_cur[at] = cur;
                    }
                    break;
                }
            }
        }
    }
}

// 3-D prefix sum of the dirty tiles (sat = number of dirty tiles in the box
// from the origin to the tile), one thread per line per axis; the x pass
// also clears the dirty marks for the next detection
__global__ void k_sat_x(uint8_t *dirty, uint32_t *sat, int ntx, int nty, int ntz) {
    const i64 lines = (i64)nty * ntz;
    for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < lines; t += (i64)gridDim.x * blockDim.x) {
        uint32_t run = 0;
        for (int x = 0; x < ntx; x++) {
            const i64 i = t * ntx + x;
            run += dirty[i];
            dirty[i] = 0;
            sat[i] = run;
        }
    }
}
__global__ void k_sat_yz(uint32_t *sat, int ntx, int nty, int ntz, int axis) {
    const i64 lines = axis == 1 ? (i64)ntx * ntz : (i64)ntx * nty;
    const int n = axis == 1 ? nty : ntz;
    const i64 step = axis == 1 ? (i64)ntx : (i64)ntx * nty;
    for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < lines; t += (i64)gridDim.x * blockDim.x) {
        const i64 base = axis == 1 ? (t % ntx) + (t / ntx) * (i64)ntx * nty : t;
        uint32_t run = 0;
        for (int k = 0; k < n; k++) {
            run += sat[base + k * step];
            sat[base + k * step] = run;
        }
    }
}
// a walk's tile box: x0 x1 y0 y1 z0 z1 in 10-bit fields, bit 63 = known
// (a box with x0 > x1 is empty: the walk reads nothing that can change)
constexpr unsigned long long kBoxKnown = 1ull << 63;
__device__ __forceinline__ unsigned long long box_pack(int x0, int x1, int y0, int y1, int z0, int z1) {
    return kBoxKnown | (unsigned long long)x0 | ((unsigned long long)x1 << 10) | ((unsigned long long)y0 << 20) |
           ((unsigned long long)y1 << 30) | ((unsigned long long)z0 << 40) | ((unsigned long long)z1 << 50);
}
struct TileSat {
    const uint32_t *sat;
    int ntx, nty, ntz;
};
__device__ __forceinline__ uint32_t sat_at(const TileSat &T, int x, int y, int z) {
    if (x < 0 || y < 0 || z < 0) return 0u;
    return T.sat[x + (i64)T.ntx * (y + (i64)T.nty * z)];
}
// dirty tiles in a known box (0 for an empty box)
__device__ __forceinline__ uint32_t box_dirty(const TileSat &T, unsigned long long b) {
    const int x0 = (int)(b & 1023), x1 = (int)((b >> 10) & 1023), y0 = (int)((b >> 20) & 1023),
              y1 = (int)((b >> 30) & 1023), z0 = (int)((b >> 40) & 1023), z1 = (int)((b >> 50) & 1023);
    if (x0 > x1) return 0u;
    return sat_at(T, x1, y1, z1) - sat_at(T, x0 - 1, y1, z1) - sat_at(T, x1, y0 - 1, z1) - sat_at(T, x1, y1, z0 - 1) +
           sat_at(T, x0 - 1, y0 - 1, z1) + sat_at(T, x0 - 1, y1, z0 - 1) + sat_at(T, x1, y0 - 1, z0 - 1) -
           sat_at(T, x0 - 1, y0 - 1, z0 - 1);
}

// start tetrahedron (anchor offset, slot) of coface j of a triangle of slot
// sl, from four immediates (9 bits per (sl, j): dx+1, dy+1, dz+1, slot)
// instead of a table read whose index differs across the warp
__host__ __device__ constexpr unsigned long long cof_word(int w) {
    unsigned long long r = 0;
    for (int i = 0; i < 7; i++) {
        const int q = w * 7 + i;
        if (q >= 24) break;
        const signed char *t = cxt::TOPO_FACE_COF[q / 2][q % 2];
        r |= (unsigned long long)((t[0] + 1) | ((t[1] + 1) << 2) | ((t[2] + 1) << 4) | (t[3] << 6)) << (9 * i);
    }
    return r;
}
__device__ __forceinline__ void face_cof_start(int sl, int j, int &dx, int &dy, int &dz, int &ts) {
    constexpr unsigned long long W0 = cof_word(0), W1 = cof_word(1), W2 = cof_word(2), W3 = cof_word(3);
    const int q = 2 * sl + j, w = q / 7, i = q - 7 * w;
    const unsigned long long word = w == 0 ? W0 : (w == 1 ? W1 : (w == 2 ? W2 : W3));
    const unsigned v = (unsigned)(word >> (9 * i)) & 511u;
    dx = (int)(v & 3u) - 1;
    dy = (int)((v >> 2) & 3u) - 1;
    dz = (int)((v >> 4) & 3u) - 1;
    ts = (int)(v >> 6);
}
static_assert(cxt::TOPO_FACE_NCOF[0] == 2 && cxt::TOPO_FACE_NCOF[5] == 2 && cxt::TOPO_FACE_NCOF[11] == 2,
              "every triangle slot has two cofaces");

// get_false_as_vpath (main_3d.cu:4540-4610) with is_false: for each original
// 2-saddle triangle, its cofaces in search order; along each one's original
// ascending path, the first tetrahedron whose decompressed pairing differs is
// recorded, for the first coface that has one.  Done in two kernels for
// parallelism: (2-saddle, coface) walks (res = the first differing
// tetrahedron, -1 none, -2 no coface), then one thread per 2-saddle keeps the
// first coface in search order that has one.  Walk lengths vary a lot, so a lane whose walk ends takes the next
// walk of its warp's contiguous range of walks instead of idling until the
// warp's longest walk ends (one step per loop turn; the warp refills its free
// lanes together, without atomics).
//
// Walk cache: a walk's result depends only on the decompressed pairing of the
// tetrahedra it visited (up to its first differing one, or to its end), and
// those sit at anchors inside the box of tiles the walk recorded.  A walk
// whose box holds no tile re-paired since the last detection keeps its
// result and is not walked again.
// Walks are handed out in chunks of kWalkChunk by a ticket (*ticket, zero at
// launch): a warp's idle lanes take the next walks of its chunk, then of the
// next free chunk of the whole list, so warps that meet long walks do not hold
// the kernel's end while others sit idle (one atomic per chunk, not per refill).
__global__ void k_path_as_walk(Grid g, const i64 *sad2, const unsigned long long *nsad, const uint32_t *tcP,
                               const uint32_t *tcQ, const uint8_t *succ, i64 *res, i64 cap, int *err,
                               unsigned long long *wbox, TileSat T, unsigned long long *ticket) {
    constexpr i64 kWalkChunk = 64;
    const i64 n = 2 * (i64)*nsad;
    const unsigned full = 0xffffffffu, lane = threadIdx.x & 31u;
    i64 pos = 0, end = 0;  // the warp's current chunk (the same in every lane)
    i64 item = -1, steps = 0;
    int x = 0, y = 0, z = 0, s = 0;
    int bx0 = 0, bx1 = 0, by0 = 0, by1 = 0, bz0 = 0, bz1 = 0;  // tile box of the current walk
    bool drained = false;
    while (true) {
        const unsigned want = __ballot_sync(full, item < 0 && !drained);
        if (want) {
            if (pos >= end) {  // the warp's chunk is used up: take the next one
                unsigned long long b0 = 0;
                if (lane == 0) b0 = atomicAdd(ticket, (unsigned long long)kWalkChunk);
                pos = (i64)__shfl_sync(full, b0, 0);
                end = min(n, pos + kWalkChunk);
            }
            const i64 my = pos + __popc(want & ((1u << lane) - 1u));
            if (item < 0 && !drained) {
                if (pos >= n) {
                    drained = true;  // no walk is left anywhere
                } else if (my < end) {
                    const unsigned long long b = wbox[my];
                    if (!(b & kBoxKnown) || box_dirty(T, b) != 0u) {
                        item = my;
                        steps = 0;
                        const i64 code = sad2[my >> 1];
                        const int j = (int)(my & 1);
                        int vx, vy, vz, dx, dy, dz;
                        decode_v(g, code / 12, vx, vy, vz);
                        face_cof_start((int)(code % 12), j, dx, dy, dz, s);
                        x = vx + dx;
                        y = vy + dy;
                        z = vz + dz;
                        bx0 = bx1 = x >> kTileShift;
                        by0 = by1 = y >> kTileShift;
                        bz0 = bz1 = z >> kTileShift;
                        const bool ok = cell_ok(g, x, y, z, 1, 1, 1);
                        if (!ok) {  // no coface there: static, never walked again
                            res[item] = -2;
                            wbox[item] = box_pack(1, 0, 0, 0, 0, 0);
                            item = -1;
                        }
                    }
                }  // else: past this chunk's end, the next refill takes a new chunk
            }
            pos = min(pos + (i64)__popc(want), end);
        }
        if (__all_sync(full, item < 0 && drained)) break;
        if (item >= 0) {  // one step of the walk
            const i64 ci = x + (i64)y * g.W + (i64)z * g.WH;
            const uint32_t wp = tcP[ci], wq = tcQ[ci];
            const int s8 = succ[ci * 8 + s];
            const int p = (wp >> (3 * s)) & 7;
            i64 r = 0;
            bool fin = true;
            if (p == 7) {
                r = -1;
            } else if (p != (int)((wq >> (3 * s)) & 7)) {
                r = tet_ref(g, x, y, z, s);
            } else if (s8 == 255) {
                r = -1;
            } else if (++steps > cap) {
                atomicOr(err, ERR_WALK);
                r = -1;
            } else {
                const int d = s8 / 6;
                s = s8 - 6 * d;
                x += d % 3 - 1;
                y += (d / 3) % 3 - 1;
                z += d / 9 - 1;
                bx0 = min(bx0, x >> kTileShift);
                bx1 = max(bx1, x >> kTileShift);
                by0 = min(by0, y >> kTileShift);
                by1 = max(by1, y >> kTileShift);
                bz0 = min(bz0, z >> kTileShift);
                bz1 = max(bz1, z >> kTileShift);
                fin = false;
            }
            if (fin) {
                res[item] = r;
                wbox[item] = box_pack(bx0, bx1, by0, by1, bz0, bz1);
                item = -1;
            }
        }
    }
}
__global__ void k_path_as_pick(Grid g, const i64 *sad2, const unsigned long long *nsad, const i64 *res, PathRec R) {
    const i64 n = (i64)*nsad;
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        const int j = res[2 * i] >= 0 ? 0 : (res[2 * i + 1] >= 0 ? 1 : -1);
        if (j < 0) continue;
        const i64 code = sad2[i];
        const i64 v = code / 12;
        const int sl = (int)(code % 12);
        int x, y, z;
        decode_v(g, v, x, y, z);
        const signed char *tc = TOPO_FACE_COF[sl][j];
        const unsigned long long at = atomicAdd(&R.n[0], 1ull);
        if ((i64)at < R.cap_as) {
            R.as_tet[at] = tet_ref(g, x + tc[0], y + tc[1], z + tc[2], tc[3]);
            R.as_cur[at] = res[2 * i + j];
        }
    }
}

// get_false_ds_vpath (main_3d.cu:4837-4959): the reference's walk never
// advances past the first vertex (dec_current_id stays at the start), so each
// endpoint's steepest-descent pairing is compared once, v1 (higher id) first.
//
// Incremental descending checks.  A 1-saddle's record depends on the
// decompressed pairing at its endpoints (its anchor, or the anchor + 1 along
// some axes).  Per anchor, C = "the tile box from the anchor's tile to the
// tile of anchor + (1,1,1) holds a tile re-paired since the last detection".
// Records of anchors with C false are kept; the anchors with C true are
// checked again (in the tiles whose box from the tile to tile + (1,1,1) is
// dirty); the first detection after the set-up checks every anchor.
__device__ __forceinline__ bool ds_anchor_dirty(const Grid &g, const TileSat &T, int x, int y, int z) {
    return box_dirty(T, box_pack(x >> kTileShift, min(x + 1, g.W - 1) >> kTileShift, y >> kTileShift,
                                 min(y + 1, g.H - 1) >> kTileShift, z >> kTileShift,
                                 min(z + 1, g.D - 1) >> kTileShift)) != 0u;
}
__global__ void k_ds_keep(Grid g, PathRec R, const unsigned long long *old_n, const unsigned long long *valid, i64 *te,
                          i64 *tv, unsigned long long *tn, i64 tcap, TileSat T) {
    if (!*valid) return;
    const i64 n = min((i64)*old_n, R.cap_ds);
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        const i64 e = R.ds_edge[i];
        int x, y, z, k;
        edge_unref(g, e, x, y, z, k);
        if (ds_anchor_dirty(g, T, x, y, z)) continue;
        const unsigned long long at = agg_slot(tn);
        if ((i64)at < tcap) {
            te[at] = e;
            tv[at] = R.ds_vert[i];
        }
    }
}
__global__ void k_ds_tiles(RuleCtx c, const unsigned long long *valid, i64 *te, i64 *tv, unsigned long long *tn,
                           i64 tcap, TileSat T) {
    const Grid &g = c.g;
    const bool all = *valid == 0;
    const i64 nt = (i64)T.ntx * T.nty * T.ntz;
    for (i64 t = blockIdx.x; t < nt; t += gridDim.x) {
        const int tx = (int)(t % T.ntx), ty = (int)((t / T.ntx) % T.nty), tz = (int)(t / ((i64)T.ntx * T.nty));
        if (!all && box_dirty(T, box_pack(tx, min(tx + 1, T.ntx - 1), ty, min(ty + 1, T.nty - 1), tz,
                                          min(tz + 1, T.ntz - 1))) == 0u)
            continue;  // the same for every thread of the block
        for (int a = threadIdx.x; a < kTile * kTile * kTile; a += blockDim.x) {
            const int x = tx * kTile + a % kTile, y = ty * kTile + (a / kTile) % kTile, z = tz * kTile + a / (kTile * kTile);
            if (x >= g.W || y >= g.H || z >= g.D) continue;
            if (!all && !ds_anchor_dirty(g, T, x, y, z)) continue;
            const i64 v = x + (i64)y * g.W + (i64)z * g.WH;
            const uint32_t m = (c.P.crit[v] >> 1) & 0x7Fu;
            if (!m) continue;
            DMTZ_FOR(7, K, {
                constexpr int k = decltype(K)::value;
                constexpr int c0 = cxt::TOPO_EDGE_V[k][0], c1 = cxt::TOPO_EDGE_V[k][1];
                if ((m >> k) & 1u) {
                    const i64 ends[2] = {v + cxt::ccx(c0) + cxt::ccy(c0) * (i64)g.W + cxt::ccz(c0) * g.WH,
                                         v + cxt::ccx(c1) + cxt::ccy(c1) * (i64)g.W + cxt::ccz(c1) * g.WH};
                    for (int j = 0; j < 2; j++) {
                        const i64 e = ends[j];
                        const int po = c.P.pv[e];
                        if (po == 15) continue;
                        if (po != c.Q.pv[e]) {
                            const unsigned long long at = agg_slot(tn);
                            if ((i64)at < tcap) {
                                te[at] = edge_ref(g, x, y, z, k);
                                tv[at] = e;
                            }
                            break;
                        }
                    }
                }
            });
        }
    }
}
__global__ void k_ds_back(PathRec R, const i64 *te, const i64 *tv, const unsigned long long *tn,
                          unsigned long long *valid) {
    const i64 n = min((i64)*tn, R.cap_ds);
    const i64 tid = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    for (i64 i = tid; i < n; i += (i64)gridDim.x * blockDim.x) {
        R.ds_edge[i] = te[i];
        R.ds_vert[i] = tv[i];
    }
    if (tid == 0) {
        R.n[1] = *tn;
        *valid = 1ull;
    }
}

// Strict descending check (dmtz_opts.strict_separatrices; no counterpart in
// the reference).  get_false_ds_vpath compares each endpoint's pairing only
// at the first vertex of its path (see above); this check walks the whole
// original descending path of each endpoint of every original 1-saddle (v1,
// the higher id, first; the walk follows the original steepest-descent
// pairing to a minimum) and records the first vertex whose decompressed
// pairing differs, in the same record format, so fix_ds_vpath's rule
// (rule_ds_path) repairs it.  With no record left, every original descending
// separatrix is a decompressed one vertex for vertex, so the descending
// labels of all 1-saddle endpoints agree.
__device__ __forceinline__ i64 dir_offset(const Grid &g, int d) {
    i64 o = 0;
#pragma unroll
    for (int i = 0; i < 14; i++)
        if (d == i) o = g.doff[i];
    return o;
}
// Items are the original 1-saddles (the list of k_crit_list<1, 7>); one lane
// walks one item's first endpoint's path, then, if that is clean, the
// second's, and idle lanes take new items from chunks of 64 handed out by a
// ticket (*ticket, zero at launch): walks are long and uneven, and a lane that
// finished does not wait for the warp's longest walk.
__global__ void k_ds_strict(RuleCtx c, PathRec R, const i64 *sad1, const unsigned long long *nsad1, i64 step_cap,
                            unsigned long long *ticket) {
    const Grid &g = c.g;
    constexpr i64 kChunk = 64;
    // corners (dx + 2 dy + 4 dz) of edge family k, higher id first: bits 6k .. 6k+5
    constexpr uint64_t kEnds = []() {
        uint64_t e = 0;
        for (int k = 0; k < 7; k++)
            e |= (uint64_t)(cxt::TOPO_EDGE_V[k][0] | (cxt::TOPO_EDGE_V[k][1] << 3)) << (6 * k);
        return e;
    }();
    const i64 n = min((i64)*nsad1, R.cap_ds);
    const unsigned full = 0xffffffffu, lane = threadIdx.x & 31u;
    i64 pos = 0, end = 0, item = -1, steps = 0, u = 0, second = 0, edge = 0;
    bool first = true, drained = false;
    while (true) {
        const unsigned want = __ballot_sync(full, item < 0 && !drained);
        if (want) {
            if (pos >= end) {  // the warp's chunk is used up: take the next one
                unsigned long long b0 = 0;
                if (lane == 0) b0 = atomicAdd(ticket, (unsigned long long)kChunk);
                pos = (i64)__shfl_sync(full, b0, 0);
                end = min(n, pos + kChunk);
            }
            const i64 my = pos + __popc(want & ((1u << lane) - 1u));
            if (item < 0 && !drained) {
                if (pos >= n) {
                    drained = true;
                } else if (my < end) {
                    const i64 code = sad1[my], a = code / 7;
                    const int k = (int)(code - 7 * a);
                    int x, y, z;
                    decode_v(g, a, x, y, z);
                    const int ends = (int)((kEnds >> (6 * k)) & 63u), c0 = ends & 7, c1 = ends >> 3;
                    u = a + (c0 & 1) + ((c0 >> 1) & 1) * (i64)g.W + (c0 >> 2) * g.WH;
                    second = a + (c1 & 1) + ((c1 >> 1) & 1) * (i64)g.W + (c1 >> 2) * g.WH;
                    edge = edge_ref(g, x, y, z, k);
                    item = my;
                    first = true;
                    steps = 0;
                }
            }
            pos = min(pos + (i64)__popc(want), end);
        }
        if (__all_sync(full, item < 0 && drained)) break;
        if (item >= 0) {  // one step of the current endpoint's walk
            const int po = c.P.pv[u];
            if (po == 15) {  // an original minimum: this endpoint's path is clean
                if (first) {
                    first = false;
                    u = second;
                    steps = 0;
                } else {
                    item = -1;
                }
            } else if (po != c.Q.pv[u]) {
                const unsigned long long at = agg_slot(R.n + 1);
                if ((i64)at < R.cap_ds) {
                    R.ds_edge[at] = edge;
                    R.ds_vert[at] = u;
                }
                item = -1;
            } else if (++steps > step_cap) {  // a cycle: not a gradient
                atomicOr(c.err, ERR_WALK);
                item = -1;
            } else {
                u += dir_offset(g, po);
            }
        }
    }
}

__global__ void k_fix_path(RuleCtx c, PathRec R) {
    const i64 na = min((i64)R.n[0], R.cap_as), nd = min((i64)R.n[1], R.cap_ds);
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < na + nd; i += (i64)gridDim.x * blockDim.x) {
        if (i < na) rule_as_path(c, R.as_cur[i]);
        else rule_ds_path(c, R.ds_vert[i - na]);
    }
}

// --------------------------------------------------------------- value update
// applyDeltaBuffer1 (main_3d.cu:1122-1164) on the requested vertices only.
// The delta is what the reference's buffer holds: get_delta(v), with the
// buffer's "no request" sentinel -2000*range (a request whose delta is not
// above the sentinel leaves the buffer unchanged under edit_type 0).
__global__ void k_apply(RuleCtx c, double range, int preserve_type, int update, uint8_t *changed, double *delta_out) {
    const i64 n = (i64)*c.reqn;
    const double sentinel = -2000.0 * range;
    const double tiny = 1e-15 * range;
    double *g = const_cast<double *>(c.gv);
    int *cnt = const_cast<int *>(c.cnt);
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n && i < c.reqcap; i += (i64)gridDim.x * blockDim.x) {
        const i64 v = c.reqlist[i];
        c.reqbits[v >> 5] = 0;  // every bit of this word belongs to listed vertices
        const double d = get_delta(c, v);
        const bool req = c.edit_type == 0 ? (d > sentinel) : (d != sentinel);
        if (delta_out) delta_out[v] = req ? d : sentinel;
        if (!req || !update) continue;
        const double f = c.f[v];
        const double gv = g[v];
        const int cv = cnt[v];
        const double lowb = __dsub_rn(f, c.bound);
        if (preserve_type == 0 && fabs(d) > tiny && cv < 5 && fabs(__dsub_rn(f, __dadd_rn(gv, d))) <= c.bound) {
            g[v] = __dadd_rn(gv, d);
            cnt[v] = cv + 1;
            if (c.progress) *c.progress = 1ull;
        } else {
            cnt[v] = 6;
            g[v] = lowb;
            if (c.progress && (cv != 6 || gv != lowb)) *c.progress = 1ull;
        }
        if (changed) changed[v] = 1;
    }
}

// ------------------------------------------------------------- stall breaker
// A round whose update changes no value and no edit counter leaves the state
// as it was, so the reference's loop repeats it forever (main_3d.cu:6784 has
// no exit for this; e.g. a false extremum no rule addresses, or requests on
// vertices already at f - bound).  With break_stalls, such a round instead
// sets every vertex within `radius` (per axis) of a vertex of a remaining
// mismatched cell -- or of a separatrix record's tetrahedron or vertex -- back
// to its original value, which is always within the bound, and requests it so
// that the next re-pairing covers it; then the loop goes on.  Rounds that make
// progress are never touched, so runs that converge under the reference's
// rules give the reference's output.
//
// The region is built in spare bits of the per-vertex `changed` bytes (bit 0
// is the edit mark): seeds get bit 1, three separable line dilations grow it
// to the box of half-width `radius` around every seed, and k_snap_mask resets
// the region and clears the bits.  Seed writers all store (bit 0 | 2) to the
// byte, and bit 0 does not change meanwhile, so unordered writes agree.
constexpr uint8_t kSnapSeed = 2, kSnapGrow = 4;
__device__ __forceinline__ void seed_vertex(const Grid &g, uint8_t *m, i64 v) {
    if (v >= 0 && v < g.V) m[v] = (uint8_t)(m[v] | kSnapSeed);
}
__global__ void k_seed_cells(Grid g, CpLists L, uint8_t *m) {
    const i64 n0 = min((i64)L.n[0], L.cap[0]), n1 = min((i64)L.n[1], L.cap[1]), n2 = min((i64)L.n[2], L.cap[2]),
              n3 = min((i64)L.n[3], L.cap[3]);
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n0 + n1 + n2 + n3; i += (i64)gridDim.x * blockDim.x) {
        i64 vs[4] = {-1, -1, -1, -1};
        if (i < n0) {
            vs[0] = L.l[0][i];
        } else if (i < n0 + n1) {
            edge_verts(g, L.l[1][i - n0], vs[0], vs[1]);
        } else if (i < n0 + n1 + n2) {
            tri_verts(g, L.l[2][i - n0 - n1], vs[0], vs[1], vs[2]);
        } else {
            tet_verts(g, L.l[3][i - n0 - n1 - n2], vs[0], vs[1], vs[2], vs[3]);
        }
        for (int k = 0; k < 4; k++) seed_vertex(g, m, vs[k]);
    }
}
__global__ void k_seed_paths(Grid g, PathRec R, uint8_t *m) {
    const i64 na = min((i64)R.n[0], R.cap_as), nd = min((i64)R.n[1], R.cap_ds);
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < na + nd; i += (i64)gridDim.x * blockDim.x) {
        i64 vs[4] = {-1, -1, -1, -1};
        if (i < na) tet_verts(g, R.as_cur[i], vs[0], vs[1], vs[2], vs[3]);
        else vs[0] = R.ds_vert[i - na];
        for (int k = 0; k < 4; k++) seed_vertex(g, m, vs[k]);
    }
}
__global__ void k_seed_walls(Grid g, WallRec W, uint8_t *m) {
    const i64 n = min((i64)*W.n, W.cap);
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        i64 a, b;
        edge_verts(g, W.edge[i], a, b);
        seed_vertex(g, m, a);
        seed_vertex(g, m, b);
    }
}
// one thread per line along `axis` (0 = x, 1 = y, 2 = z): every position
// within `radius` of a seed of the line becomes a seed
__global__ void k_dilate_axis(Grid g, uint8_t *m, int axis, int radius) {
    const int n = axis == 0 ? g.W : axis == 1 ? g.H : g.D;
    const i64 step = axis == 0 ? 1 : axis == 1 ? (i64)g.W : g.WH;
    const i64 lines = g.V / n;
    for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < lines; t += (i64)gridDim.x * blockDim.x) {
        i64 base;
        if (axis == 0) base = t * g.W;                                  // t = y + H z
        else if (axis == 1) base = (t % g.W) + (t / g.W) * g.WH;        // t = x + W z
        else base = t;                                                  // t = x + W y
        int last = -radius - 1;
        for (int i = 0; i < n; i++) {
            const uint8_t b = m[base + i * step];
            if (b & kSnapSeed) last = i;
            if (i - last <= radius) m[base + i * step] = (uint8_t)(b | kSnapGrow);
        }
        int next = n + radius + 1;
        for (int i = n - 1; i >= 0; i--) {
            uint8_t b = m[base + i * step];
            if (b & kSnapSeed) next = i;
            if (next - i <= radius) b |= kSnapGrow;
            m[base + i * step] = (uint8_t)((b & 1) | ((b & kSnapGrow) ? kSnapSeed : 0));
        }
    }
}
__global__ void k_snap_mask(RuleCtx c, uint8_t *m) {
    double *gv = const_cast<double *>(c.gv);
    for (i64 v = (i64)blockIdx.x * blockDim.x + threadIdx.x; v < c.g.V; v += (i64)gridDim.x * blockDim.x) {
        const uint8_t b = m[v];
        if (!(b & kSnapSeed)) continue;
        m[v] = (uint8_t)(b & 1);
        if (gv[v] != c.f[v]) {
            gv[v] = c.f[v];
            m[v] = 1;
            lower(c, v);  // a request: the re-pairing looks here
        }
    }
}
// the request bits of the listed vertices back to 0 (k_apply does this for
// the vertices it updates; snapped vertices are only re-paired)
__global__ void k_clear_req(const i64 *reqlist, const unsigned long long *n, i64 cap, uint32_t *reqbits) {
    const i64 m = min((i64)*n, cap);
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (i64)gridDim.x * blockDim.x)
        reqbits[reqlist[i] >> 5] = 0;
}

// filter_vertices / _edges / _faces / _tetrahedras (main_3d.cu:2405-2490):
// every vertex of every original critical cell goes to f - bound
__global__ void k_filter(Grid g, const uint32_t *crit_o, const double *f, double *gv, double bound) {
    i64 v = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= g.V) return;
    uint32_t m = crit_o[v];
    if (!m) return;
    int x, y, z;
    decode_v(g, v, x, y, z);
    uint32_t corners = 0;
    if (m & 1u) corners |= 1u;
    for (int k = 0; k < 7; k++)
        if (m & (1u << (1 + k))) corners |= (1u << TOPO_EDGE_V[k][0]) | (1u << TOPO_EDGE_V[k][1]);
    for (int s = 0; s < 12; s++)
        if (m & (1u << (8 + s)))
            corners |= (1u << TOPO_FACE_V[s][0]) | (1u << TOPO_FACE_V[s][1]) | (1u << TOPO_FACE_V[s][2]);
    for (int s = 0; s < 6; s++)
        if (m & (1u << (20 + s)))
            corners |= (1u << TOPO_TET_V[s][0]) | (1u << TOPO_TET_V[s][1]) | (1u << TOPO_TET_V[s][2]) |
                       (1u << TOPO_TET_V[s][3]);
    while (corners) {
        const int c8 = __ffs(corners) - 1;
        corners &= corners - 1;
        const i64 u = v + g.coff[c8];
        gv[u] = __dsub_rn(f[u], bound);  // same value from every writer
    }
}

// --------------------------------------------------------------- manifold labels
// Descending manifold label of a vertex: the minimum its steepest-descent path
// (vertex -> other endpoint of its paired edge, processVertices'
// pairing) reaches.  Ascending label of a tetrahedron: the maximum (unpaired
// tetrahedron) its ascending path (is_false's walk, main_3d.cu:4437-4497)
// reaches, or -1 when the path leaves through the boundary.  Both by pointer
// jumping: lab <- lab[lab] until nothing changes.
__global__ void k_desc_init(Grid g, const uint8_t *pv, i64 *lab) {
    for (i64 v = (i64)blockIdx.x * blockDim.x + threadIdx.x; v < g.V; v += (i64)gridDim.x * blockDim.x) {
        const int d = pv[v];
        lab[v] = d == 15 ? v : v + g.doff[d];
    }
}
__global__ void k_asc_init(Grid g, const uint32_t *tcode, const uint8_t *succ, i64 *lab) {
    for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < 6 * g.V; t += (i64)gridDim.x * blockDim.x) {
        const i64 v = t / 6;
        const int ts = (int)(t - 6 * v);
        int x, y, z;
        decode_v(g, v, x, y, z);
        if (!cell_ok(g, x, y, z, 1, 1, 1)) {
            lab[t] = -2;  // no such tetrahedron
            continue;
        }
        if (((tcode[v] >> (3 * ts)) & 7) == 7) {
            lab[t] = t;  // a maximum
            continue;
        }
        const int s8 = succ[v * 8 + ts];
        if (s8 == 255) {
            lab[t] = -1;  // leaves through the boundary
            continue;
        }
        const int d = s8 / 6;
        const i64 nv = v + (d % 3 - 1) + (i64)((d / 3) % 3 - 1) * g.W + (i64)(d / 9 - 1) * g.WH;
        lab[t] = nv * 6 + (s8 - 6 * d);
    }
}
__global__ void k_jump(i64 *lab, i64 n, int *changed) {
    int any = 0;
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        const i64 l = lab[i];
        if (l < 0) continue;
        const i64 ll = lab[l];
        if (ll != l) {
            lab[i] = ll;
            any = 1;
        }
    }
    if (__syncthreads_or(any) && threadIdx.x == 0) atomicOr(changed, 1);
}
// reference ids of the labels
__global__ void k_desc_out(Grid g, const i64 *lab, int32_t *out) {
    for (i64 v = (i64)blockIdx.x * blockDim.x + threadIdx.x; v < g.V; v += (i64)gridDim.x * blockDim.x)
        out[v] = (int32_t)lab[v];
}
__global__ void k_asc_out(Grid g, const i64 *lab, int32_t *out) {
    for (i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x; t < 6 * g.V; t += (i64)gridDim.x * blockDim.x) {
        const i64 v = t / 6;
        const int ts = (int)(t - 6 * v);
        int x, y, z;
        decode_v(g, v, x, y, z);
        if (!cell_ok(g, x, y, z, 1, 1, 1)) continue;
        const i64 l = lab[t];
        int32_t r = -1;
        if (l >= 0) {
            const i64 lv = l / 6;
            int lx, ly, lz;
            decode_v(g, lv, lx, ly, lz);
            r = (int32_t)tet_ref(g, lx, ly, lz, (int)(l - 6 * lv));
        }
        out[tet_ref(g, x, y, z, ts)] = r;
    }
}

// exact min / max of a field through its order keys
__global__ void k_minmax(const double *a, i64 n, unsigned long long *kmin, unsigned long long *kmax) {
    unsigned long long lo = ~0ull, hi = 0ull;
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        const unsigned long long k = okey(a[i]);
        lo = k < lo ? k : lo;
        hi = k > hi ? k : hi;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long l2 = __shfl_xor_sync(0xffffffffu, lo, o), h2 = __shfl_xor_sync(0xffffffffu, hi, o);
        lo = l2 < lo ? l2 : lo;
        hi = h2 > hi ? h2 : hi;
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(kmin, lo);
        atomicMax(kmax, hi);
    }
}

__global__ void k_count_u8(const uint8_t *a, i64 n, unsigned long long *out) {
    unsigned long long c = 0;
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) c += a[i] != 0;
    for (int off = 16; off > 0; off >>= 1) c += __shfl_down_sync(0xffffffffu, c, off);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}
__global__ void k_fill_i32(int *p, int val, i64 n) {
    i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = val;
}
__global__ void k_check_finite(const double *a, i64 n, int *bad) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x)
        if (!isfinite(a[i])) atomicOr(bad, 1);
}

}  // namespace dmtz

// =============================================================================
// host side
// =============================================================================
// ----------------------------------------------------- decompression model
// SZ-style error-bounded quantisation of the original field, done on the GPU
// (the reference runs an external compressor and reads its output back,
// main_3d.cu:6331-6356): g = fmin + 2 eps * rint((f - fmin) / (2 eps)); then a
// fraction `frac` of the vertices gets extra uniform noise in [-eps, eps); then
// g is clamped into [f - eps, f + eps].  Random numbers are a counter-based
// hash of (seed, vertex, stream): the splitmix64 finaliser, 53 bits to [0, 1).
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ double unit_rand(uint64_t seed, i64 v, int k) {
    const uint64_t h = mix64(seed + 0x9E3779B97F4A7C15ull * (uint64_t)(2 * v + k + 1));
    return (double)(h >> 11) * 0x1.0p-53;
}
__global__ void k_quantize(i64 V, const double *f, double *g, double fmn, double eps, double frac, uint64_t seed) {
    const double w = __dmul_rn(2.0, eps);
    for (i64 v = (i64)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (i64)gridDim.x * blockDim.x) {
        const double fv = f[v];
        double q = w > 0.0 ? __dadd_rn(fmn, __dmul_rn(w, rint(__ddiv_rn(__dsub_rn(fv, fmn), w)))) : fv;
        if (unit_rand(seed, v, 0) < frac)
            q = __dadd_rn(q, __dmul_rn(eps, __dsub_rn(__dmul_rn(2.0, unit_rand(seed, v, 1)), 1.0)));
        const double lo = __dsub_rn(fv, eps), hi = __dadd_rn(fv, eps);
        g[v] = q < lo ? lo : (q > hi ? hi : q);
    }
}

// ----------------------------------------------------- learned-proposal glue
// Network input per vertex (layout in cnn.cuh) and the mismatch byte mm[v]
// (criticality of v's own cells differs between the two gradients).
__global__ void k_features(Grid g, const double *f, const double *gv, const uint32_t *critP, const uint32_t *critQ,
                           double bound, __nv_bfloat16 *feat, uint8_t *mm) {
    for (i64 v = (i64)blockIdx.x * blockDim.x + threadIdx.x; v < g.V; v += (i64)gridDim.x * blockDim.x) {
        int x, y, z;
        decode_v(g, v, x, y, z);
        const double fv = f[v];
        const bool mis = critP[v] != critQ[v];
        mm[v] = mis;
        float c[16];
        c[0] = bound > 0 ? fminf(fmaxf((float)((gv[v] - fv) / bound), -1.f), 1.f) : 0.f;
        c[1] = mis ? 1.f : 0.f;
#pragma unroll
        for (int k = 0; k < 14; k++) {
            const int nx = x + TOPO_DIRS[k][0], ny = y + TOPO_DIRS[k][1], nz = z + TOPO_DIRS[k][2];
            float cv = 0.f;
            if (bound > 0 && nx >= 0 && nx < g.W && ny >= 0 && ny < g.H && nz >= 0 && nz < g.D)
                cv = tanhf((float)((f[v + g.doff[k]] - fv) / (4.0 * bound)));
            c[2 + k] = cv;
        }
        uint32_t packed[8];
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const __nv_bfloat162 b = __floats2bfloat162_rn(c[2 * k], c[2 * k + 1]);
            packed[k] = *reinterpret_cast<const uint32_t *>(&b);
        }
        uint4 *dst = reinterpret_cast<uint4 *>(feat + v * 16);
        dst[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
        dst[1] = make_uint4(packed[4], packed[5], packed[6], packed[7]);
    }
}
// dst[v] = max of src over v + k*step, |k| <= 2, along one axis (in-grid)
__global__ void k_dilate(Grid g, int axis, const uint8_t *src, uint8_t *dst) {
    const i64 step = axis == 0 ? 1 : axis == 1 ? (i64)g.W : g.WH;
    for (i64 v = (i64)blockIdx.x * blockDim.x + threadIdx.x; v < g.V; v += (i64)gridDim.x * blockDim.x) {
        int c[3];
        decode_v(g, v, c[0], c[1], c[2]);
        const int n = axis == 0 ? g.W : axis == 1 ? g.H : g.D;
        uint8_t m = 0;
        for (int k = -2; k <= 2; k++) {
            const int q = c[axis] + k;
            if (q >= 0 && q < n) m |= src[v + k * step];
        }
        dst[v] = m;
    }
}
// Proposal at active vertices: g <- f + bound * tanh(o) where that lowers g by
// at least min_drop (absolute; the network's min_drop x bound); a value that
// the reference's own bound test |f - g| <= bound would reject becomes
// f - bound, the value the reference falls back to (main_3d.cu:1133-1141).
// the proposal's edits also go to the request list, so that only the bricks
// around them are re-paired afterwards
__global__ void k_propose(i64 V, const double *f, double *gv, const float *o, const uint8_t *active, double bound,
                          double min_drop, uint8_t *changed, i64 *reqlist, unsigned long long *reqn) {
    for (i64 v = (i64)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (i64)gridDim.x * blockDim.x) {
        if (!active[v]) continue;
        const double fv = f[v], old = gv[v];
        const double p = __dadd_rn(fv, __dmul_rn(bound, (double)tanhf(o[v])));
        if (!(old - p >= min_drop)) continue;  // keep g unless the proposal lowers it enough
        double nv = p;
        if (fabs(__dsub_rn(fv, nv)) > bound) nv = __dsub_rn(fv, bound);
        if (nv != old) {
            gv[v] = nv;
            changed[v] = 1;
            reqlist[agg_slot(reqn)] = v;
        }
    }
}

struct DevField {
    uint64_t *key = nullptr;
    uint16_t *low = nullptr;
    uint8_t *pv = nullptr;
    uint32_t *ea2 = nullptr;
    uint16_t *fp3 = nullptr;
    uint32_t *fa3 = nullptr;
    uint32_t *eup = nullptr;
    uint32_t *fup = nullptr;
    uint32_t *crit = nullptr;
    uint32_t *tcode = nullptr;
};

struct dmtz_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;      // copies that overlap the context stream's work
    cudaEvent_t side_done = nullptr;
    std::string err;
    // sized buffers
    i64 capV = 0, capE = 0, capF = 0, capT = 0, capB = 0;
    double *f = nullptr, *g = nullptr;
    DevField P, Q;
    int *cnt = nullptr;
    uint32_t *reqbits = nullptr;
    i64 *reqlist = nullptr;
    // Mismatch lists and separatrix records.  Sized for the counts that occur,
    // not for every cell: the mismatch lists start at list_frac x cells (at
    // least list_min entries, at most all cells) and grow when a scan
    // overflows them; the path records and the 2-saddle list are sized from
    // the original gradient's saddle counts, which bound them.
    i64 *lists[4] = {nullptr, nullptr, nullptr, nullptr};
    i64 capL[4] = {0, 0, 0, 0};
    double list_frac = 1.0 / 16;
    i64 list_min = 1 << 20;
    i64 *as_tet = nullptr, *as_cur = nullptr, *ds_edge = nullptr, *ds_vert = nullptr;
    i64 *ds_tmp_edge = nullptr, *ds_tmp_vert = nullptr;  // descending records being rebuilt, capDST each
    i64 capDST = 0;
    i64 capAS = 0, capDS = 0, capSad2 = 0;
    uint8_t *succ = nullptr;  // original ascending-path successor of each tetrahedron
    uint32_t *brick_flags = nullptr;  // per brick (a byte each, four to a word): radius bits of the next sweep
    uint8_t *brick_fresh = nullptr;   // per brick: re-paired by the current round's criticality pass
    int inc_scan = 0;                 // repairs rebuild the mismatch lists incrementally (see k_list_keep)
    int strict_ds = 0;                // descending separatrix checks walk whole paths (k_ds_strict)
    i64 *list_tmp[4] = {nullptr, nullptr, nullptr, nullptr};  // rebuilt mismatch lists, capL entries each
    uint32_t *brick_list = nullptr;   // compacted lists per radius, capB entries each
    unsigned long long *brick_n = nullptr;  // their lengths
    i64 *sad2 = nullptr;      // original 2-saddle triangles
    i64 *sad1 = nullptr;      // original 1-saddle edges (strict descending checks only)
    i64 capSad1 = 0;
    i64 *as_res = nullptr;    // per (2-saddle, coface) walk results, 2 x capSad2
    // walk cache: per walk, the box of 16^3-anchor tiles its last walk visited
    // (walk_box); per tile, whether the decompressed gradient was recomputed
    // there since the last detection (tile_dirty) and its 3-D prefix sum
    unsigned long long *walk_box = nullptr;
    uint8_t *tile_dirty = nullptr;
    uint32_t *tile_sat = nullptr;
    i64 capWB = 0, capTile = 0;
    int ntx = 0, nty = 0, ntz = 0;
    i64 *wall_sad = nullptr, *wall_edge = nullptr;  // wall records (preserve_connectors = 1), capWall each
    i64 *wall_next[2] = {nullptr, nullptr};          // 2-saddles handed to the next search tier
    i64 capWall = 0;
    i64 *wall_scratch = nullptr;  // stacks and caches of the larger wall-search tiers
    i64 capWS = 0;
    unsigned long long *counters = nullptr;  // [0..3] cp lists, [4] requests, [5,6] paths, [7] progress,
                                             // [8,9] min/max keys, [10] original 2-saddles, [12] edited
                                             // vertices, [13,14] saddle counts, [15] surface anchors,
                                             // [16] wall records, [17,18] deferred wall searches,
                                             // [20..23] rebuilt mismatch lists, [24] descending
                                             // records rebuildable, [25] their last count,
                                             // [26] rebuilt descending records
    int *errword = nullptr;
    uint8_t *changed = nullptr;
    int64_t launches = 0;  // kernels launched by the current call
    int tune_shape = 0;    // brick shape (DMTZ_SHAPES) chosen by dmtz_autotune
    int tune_bps = 32;     // sweep blocks per SM
    std::vector<dmtz_ctx *> pool;  // worker contexts of dmtz_correct_batch
    uint8_t *mm = nullptr;         // mismatch bytes of the learned proposal's features
    i64 capMM = 0;
    i64 *bnd = nullptr;            // surface anchors of the grid bndW x bndH x bndD (full sweeps)
    i64 bnd_n = 0, bnd_cap = 0;
    int bndW = 0, bndH = 0, bndD = 0;
    void *loopctl = nullptr;       // device copy of the graph loop's control block (kept: a
                                   // cudaFree per call would synchronise the whole device)
};

namespace {

dmtz_status fail(dmtz_ctx *c, dmtz_status s, const std::string &m) {
    if (c) c->err = m;
    return s;
}
#define CK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) return fail(ctx, DMTZ_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <class T>
cudaError_t dalloc(T **p, i64 n) {
    return cudaMalloc((void **)p, sizeof(T) * (size_t)std::max<i64>(n, 1));
}

void free_field(DevField &d) {
    cudaFree(d.key); cudaFree(d.low); cudaFree(d.pv); cudaFree(d.ea2); cudaFree(d.fp3);
    cudaFree(d.fa3); cudaFree(d.eup); cudaFree(d.fup); cudaFree(d.crit); cudaFree(d.tcode);
    d = DevField();
}
void free_all(dmtz_ctx *c) {
    cudaFree(c->f); cudaFree(c->g); free_field(c->P); free_field(c->Q);
    cudaFree(c->cnt); cudaFree(c->reqbits); cudaFree(c->reqlist);
    for (auto &l : c->lists) { cudaFree(l); l = nullptr; }
    for (auto &l : c->list_tmp) { cudaFree(l); l = nullptr; }
    cudaFree(c->brick_fresh);
    c->brick_fresh = nullptr;
    for (auto &k : c->capL) k = 0;
    c->capAS = c->capDS = c->capSad2 = 0;
    cudaFree(c->as_tet); cudaFree(c->as_cur); cudaFree(c->ds_edge); cudaFree(c->ds_vert);
    cudaFree(c->counters); cudaFree(c->errword); cudaFree(c->changed);
    cudaFree(c->succ); cudaFree(c->sad2); cudaFree(c->brick_flags); cudaFree(c->brick_list);
    cudaFree(c->as_res);
    c->as_res = nullptr;
    cudaFree(c->walk_box); cudaFree(c->tile_dirty); cudaFree(c->tile_sat);
    c->walk_box = nullptr; c->tile_dirty = nullptr; c->tile_sat = nullptr;
    c->capWB = c->capTile = 0;
    cudaFree(c->wall_sad); cudaFree(c->wall_edge); cudaFree(c->wall_next[0]); cudaFree(c->wall_next[1]);
    cudaFree(c->wall_scratch);
    c->wall_sad = c->wall_edge = c->wall_next[0] = c->wall_next[1] = c->wall_scratch = nullptr;
    c->capWall = c->capWS = 0;
    cudaFree(c->brick_n);
    c->brick_n = nullptr;
    cudaFree(c->sad1);
    c->sad1 = nullptr;
    c->capSad1 = 0;
    c->succ = nullptr; c->sad2 = nullptr; c->brick_flags = nullptr; c->brick_list = nullptr;
    c->f = c->g = nullptr; c->cnt = nullptr; c->reqbits = nullptr; c->reqlist = nullptr;
    c->as_tet = c->as_cur = c->ds_edge = c->ds_vert = nullptr; c->counters = nullptr;
    cudaFree(c->ds_tmp_edge); cudaFree(c->ds_tmp_vert);
    c->ds_tmp_edge = c->ds_tmp_vert = nullptr;
    c->capDST = 0;
    c->errword = nullptr; c->changed = nullptr;
    c->capV = c->capE = c->capF = c->capT = c->capB = 0;
}

dmtz_status alloc_field(dmtz_ctx *ctx, DevField &d, i64 V) {
    CK(dalloc(&d.key, V)); CK(dalloc(&d.low, V)); CK(dalloc(&d.pv, V)); CK(dalloc(&d.ea2, V));
    CK(dalloc(&d.fp3, V)); CK(dalloc(&d.fa3, V)); CK(dalloc(&d.eup, V)); CK(dalloc(&d.fup, V));
    CK(dalloc(&d.crit, V)); CK(dalloc(&d.tcode, V));
    return DMTZ_OK;
}

i64 bricks_of(const Grid &g, int shape, int &nbx, int &nby, int &nbz);

// capacity a mismatch list of a dimension with `cells` cells starts with
i64 lean_cap(const dmtz_ctx *ctx, i64 cells) {
    const i64 want = std::max<i64>(ctx->list_min, (i64)((double)cells * ctx->list_frac));
    return std::max<i64>(1, std::min<i64>(cells, want));
}

dmtz_status ensure_lists(dmtz_ctx *ctx, const Grid &g) {
    const i64 cells[4] = {g.V, g.E, g.F, g.T};
    for (int k = 0; k < 4; k++) {
        if (ctx->lists[k]) continue;
        const i64 cap = lean_cap(ctx, cells[k]);
        cudaFree(ctx->list_tmp[k]);
        ctx->list_tmp[k] = nullptr;
        CK(dalloc(&ctx->lists[k], cap));
        CK(dalloc(&ctx->list_tmp[k], cap));
        ctx->capL[k] = cap;
    }
    return DMTZ_OK;
}

dmtz_status ensure(dmtz_ctx *ctx, const Grid &g) {
    int nbx, nby, nbz;
    i64 nbr = 0;
    for (int sh = 0; sh < DMTZ_NSHAPES; sh++) nbr = std::max(nbr, bricks_of(g, sh, nbx, nby, nbz));
    if (g.V <= ctx->capV && g.E <= ctx->capE && g.F <= ctx->capF && g.T <= ctx->capT && nbr <= ctx->capB)
        return ensure_lists(ctx, g);
    free_all(ctx);
    const i64 V = g.V;
    CK(dalloc(&ctx->f, V)); CK(dalloc(&ctx->g, V));
    dmtz_status s;
    if ((s = alloc_field(ctx, ctx->P, V)) != DMTZ_OK) return s;
    if ((s = alloc_field(ctx, ctx->Q, V)) != DMTZ_OK) return s;
    CK(dalloc(&ctx->cnt, V));
    CK(dalloc(&ctx->reqbits, (V + 31) / 32 + 1));
    CK(cudaMemset(ctx->reqbits, 0, sizeof(uint32_t) * (size_t)((V + 31) / 32 + 1)));
    CK(dalloc(&ctx->reqlist, V));
    CK(dalloc(&ctx->succ, 8 * V));
    CK(dalloc(&ctx->brick_flags, (nbr + 3) / 4)); CK(dalloc(&ctx->brick_list, kRadii * nbr));
    CK(dalloc(&ctx->brick_fresh, nbr));
    CK(dalloc(&ctx->brick_n, 8));
    CK(cudaMemset(ctx->brick_flags, 0, sizeof(uint32_t) * (size_t)((nbr + 3) / 4)));
    ctx->capB = nbr;
    CK(dalloc(&ctx->counters, 32)); CK(dalloc(&ctx->errword, 1)); CK(dalloc(&ctx->changed, V));
    ctx->capV = g.V; ctx->capE = g.E; ctx->capF = g.F; ctx->capT = g.T;
    return ensure_lists(ctx, g);
}

// grow mismatch list k to hold `need` entries; its contents are lost, so the
// caller scans again
dmtz_status grow_list(dmtz_ctx *ctx, const Grid &g, int k, i64 need) {
    const i64 cells[4] = {g.V, g.E, g.F, g.T};
    const i64 cap = std::max<i64>(need, std::min<i64>(cells[k], std::max<i64>(need + need / 2, 2 * ctx->capL[k])));
    cudaFree(ctx->lists[k]);
    cudaFree(ctx->list_tmp[k]);
    ctx->lists[k] = ctx->list_tmp[k] = nullptr;
    ctx->capL[k] = 0;
    CK(dalloc(&ctx->lists[k], cap));
    CK(dalloc(&ctx->list_tmp[k], cap));
    ctx->capL[k] = cap;
    return DMTZ_OK;
}

FieldState view(const DevField &d, const double *val) {
    FieldState s;
    s.val = val; s.key = d.key; s.low = d.low; s.pv = d.pv; s.ea2 = d.ea2; s.fp3 = d.fp3;
    s.fa3 = d.fa3; s.eup = d.eup; s.fup = d.fup; s.crit = d.crit; s.tcode = d.tcode;
    return s;
}

unsigned persistent_grid();

// five passes + criticality (and mismatch lists when crit_o is given)
i64 bricks_of(const Grid &g, int shape, int &nbx, int &nby, int &nbz) {
    nbx = (g.W + DMTZ_SHAPES[shape][0] - 1) / DMTZ_SHAPES[shape][0];
    nby = (g.H + DMTZ_SHAPES[shape][1] - 1) / DMTZ_SHAPES[shape][1];
    nbz = (g.D + DMTZ_SHAPES[shape][2] - 1) / DMTZ_SHAPES[shape][2];
    return (i64)nbx * nby * nbz;
}
// brick coordinates are packed as bx | by << 11 | bz << 22
bool shape_fits(const Grid &g, int shape) {
    int nbx, nby, nbz;
    bricks_of(g, shape, nbx, nby, nbz);
    return nbx <= 2048 && nby <= 2048 && nbz <= 1024;
}

unsigned sweep_grid(const dmtz_ctx *ctx, i64 nb) {
    const unsigned cap = (unsigned)(persistent_grid() / 8) * (unsigned)ctx->tune_bps;
    return (unsigned)std::max<i64>(1, std::min<i64>(nb, cap));
}

// the five pairing passes and the criticality pass, each over its brick set
void sweep_passes(dmtz_ctx *ctx, const Grid &g, const FieldState &s, const BrickList bl[6], i64 nb_max) {
    const unsigned gr = sweep_grid(ctx, nb_max);
    cudaStream_t st = ctx->stream;
    launch_pass<PASS_VERTEX>(g, s, bl[0], gr, st);
    launch_pass<PASS_E2>(g, s, bl[1], gr, st);
    launch_pass<PASS_F3>(g, s, bl[2], gr, st);
    launch_pass<PASS_E4>(g, s, bl[3], gr, st);
    launch_pass<PASS_F5>(g, s, bl[4], gr, st);
    launch_pass<PASS_CRIT>(g, s, bl[5], gr, st);
    ctx->launches += 6;
}

// the list of the grid's surface anchors, built once per grid shape
bool surface_list(dmtz_ctx *ctx, const Grid &g) {
    if (ctx->bnd && ctx->bndW == g.W && ctx->bndH == g.H && ctx->bndD == g.D) return true;
    const i64 need = std::min<i64>(g.V, 2 * ((i64)g.W * g.H + (i64)g.W * g.D + (i64)g.H * g.D));
    if (need > ctx->bnd_cap) {
        cudaFree(ctx->bnd);
        ctx->bnd = nullptr;
        ctx->bnd_cap = 0;
        if (dalloc(&ctx->bnd, need) != cudaSuccess) {
            cudaGetLastError();
            ctx->bnd = nullptr;
            return false;
        }
        ctx->bnd_cap = need;
    }
    cudaMemsetAsync(ctx->counters + 15, 0, sizeof(unsigned long long), ctx->stream);
    k_bnd_list<<<grid_for(g.V), kBlock, 0, ctx->stream>>>(g, ctx->bnd, ctx->counters + 15);
    unsigned long long n = 0;
    cudaMemcpyAsync(&n, ctx->counters + 15, sizeof(n), cudaMemcpyDeviceToHost, ctx->stream);
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return false;
    ctx->bnd_n = (i64)n;
    ctx->bndW = g.W;
    ctx->bndH = g.H;
    ctx->bndD = g.D;
    return true;
}

// the five pairing passes and the criticality pass over a set of bricks; a
// full sweep runs the grid's surface anchors separately, in dense warps
void sweep(dmtz_ctx *ctx, const Grid &g, const FieldState &s, const BrickList &bl, i64 nb_max) {
    if (bl.list == nullptr && surface_list(ctx, g)) {
        const unsigned gr = sweep_grid(ctx, nb_max);
        cudaStream_t st = ctx->stream;
        const i64 *b = ctx->bnd;
        const i64 nbd = ctx->bnd_n;
        launch_pass<PASS_VERTEX>(g, s, bl, gr, st, 1);
        launch_bnd<PASS_VERTEX>(g, s, b, nbd, st);
        launch_pass<PASS_E2>(g, s, bl, gr, st, 1);
        launch_bnd<PASS_E2>(g, s, b, nbd, st);
        launch_pass<PASS_F3>(g, s, bl, gr, st, 1);
        launch_bnd<PASS_F3>(g, s, b, nbd, st);
        launch_pass<PASS_E4>(g, s, bl, gr, st, 1);
        launch_bnd<PASS_E4>(g, s, b, nbd, st);
        launch_pass<PASS_F5>(g, s, bl, gr, st, 1);
        launch_bnd<PASS_F5>(g, s, b, nbd, st);
        launch_pass<PASS_CRIT>(g, s, bl, gr, st, 1);
        launch_bnd<PASS_CRIT>(g, s, b, nbd, st);
        ctx->launches += 12;
        return;
    }
    const BrickList per_pass[6] = {bl, bl, bl, bl, bl, bl};
    sweep_passes(ctx, g, s, per_pass, nb_max);
}

BrickList all_bricks(const Grid &g, int shape, i64 &nb) {
    BrickList bl;
    bl.list = nullptr;
    bl.n = nullptr;
    bl.shape = shape;
    nb = bricks_of(g, shape, bl.nbx, bl.nby, bl.nbz);
    bl.dbx = make_fdiv((unsigned long long)bl.nbx);
    bl.dby = make_fdiv((unsigned long long)bl.nby);
    return bl;
}

// mismatch lists of the decompressed gradient against crit_o
void scan_mismatch(dmtz_ctx *ctx, const Grid &g, const uint32_t *crit_d, const uint32_t *crit_o, int want_saddles) {
    Lists L;
    for (int k = 0; k < 4; k++) {
        L.l[k] = ctx->lists[k];
        L.cap[k] = ctx->capL[k];
    }
    L.n = ctx->counters;
    cudaMemsetAsync(ctx->counters, 0, 4 * sizeof(unsigned long long), ctx->stream);
    k_mismatch_scan<<<persistent_grid(), kBlock, 0, ctx->stream>>>(g, crit_d, crit_o, L, want_saddles);
    ctx->launches++;
}

// full gradient of one field (and its mismatch lists when crit_o is given)
void run_pairing(dmtz_ctx *ctx, const Grid &g, const FieldState &s, const uint32_t *crit_o, int want_saddles) {
    i64 nb;
    const BrickList bl = all_bricks(g, ctx->tune_shape, nb);
    sweep(ctx, g, s, bl, nb);
    if (crit_o) scan_mismatch(ctx, g, s.crit, crit_o, want_saddles);
}

// re-pair only the bricks near the vertices the last update requested
// (ctx->reqlist), then rebuild the mismatch lists
void repair_dirty(dmtz_ctx *ctx, const Grid &g, const FieldState &s, const uint32_t *crit_o, int want_saddles) {
    int nbx, nby, nbz;
    const int shape = ctx->tune_shape;
    const i64 nb = bricks_of(g, shape, nbx, nby, nbz);
    cudaStream_t st = ctx->stream;
    cudaMemsetAsync(ctx->brick_n, 0, kRadii * sizeof(unsigned long long), st);
    k_mark_dirty<<<persistent_grid(), kBlock, 0, st>>>(g, nbx, nby, nbz, DMTZ_SHAPES[shape][0], DMTZ_SHAPES[shape][1],
                                                        DMTZ_SHAPES[shape][2], ctx->reqlist, ctx->counters + 4,
                                                        ctx->brick_flags);
    k_compact_bricks<<<persistent_grid(), kBlock, 0, st>>>(nbx, nby, nbz, ctx->brick_flags, ctx->brick_list,
                                                            ctx->capB, ctx->brick_n);
    ctx->launches += 2;
    const uint32_t *r5 = ctx->brick_list + (i64)(kRadii - 1) * ctx->capB;
    const unsigned long long *r5n = ctx->brick_n + (kRadii - 1);
    if (ctx->inc_scan) {
        cudaMemsetAsync(ctx->brick_fresh, 0, (size_t)nb, st);
        k_mark_fresh<<<persistent_grid(), kBlock, 0, st>>>(r5, r5n, ctx->brick_fresh, nbx, nby);
        ctx->launches++;
    }
    if (ctx->tile_dirty && ctx->ntx > 0) {  // the criticality pass's bricks cover every anchor re-paired
        k_mark_tiles<<<persistent_grid(), kBlock, 0, st>>>(r5, r5n, DMTZ_SHAPES[shape][0],
                                                            DMTZ_SHAPES[shape][1], DMTZ_SHAPES[shape][2], ctx->ntx,
                                                            ctx->nty, ctx->ntz, ctx->tile_dirty);
        ctx->launches++;
    }
    static const int radius[6] = {1, 2, 3, 3, 4, 5};  // per pass
    BrickList bl[6];
    for (int p = 0; p < 6; p++) {
        bl[p].list = ctx->brick_list + (i64)(radius[p] - 1) * ctx->capB;
        bl[p].n = ctx->brick_n + (radius[p] - 1);
        bl[p].nbx = nbx; bl[p].nby = nby; bl[p].nbz = nbz;
        bl[p].dbx = make_fdiv((unsigned long long)nbx);
        bl[p].dby = make_fdiv((unsigned long long)nby);
        bl[p].shape = shape;
    }
    sweep_passes(ctx, g, s, bl, nb);
    if (!ctx->inc_scan) {
        scan_mismatch(ctx, g, s.crit, crit_o, want_saddles);
        return;
    }
    Lists L, T;
    for (int k = 0; k < 4; k++) {
        L.l[k] = ctx->lists[k];
        T.l[k] = ctx->list_tmp[k];
        L.cap[k] = T.cap[k] = ctx->capL[k];
    }
    L.n = ctx->counters;
    T.n = ctx->counters + 20;
    const int sx = DMTZ_SHAPES[shape][0], sy = DMTZ_SHAPES[shape][1], sz = DMTZ_SHAPES[shape][2];
    const unsigned pg = persistent_grid();
    cudaMemsetAsync(ctx->counters + 20, 0, 4 * sizeof(unsigned long long), st);
    k_list_keep<<<pg, kBlock, 0, st>>>(g, L, T, ctx->brick_fresh, sx, sy, sz, nbx, nby);
    k_scan_fresh<<<pg, kBlock, 0, st>>>(g, s.crit, crit_o, T, r5, r5n, sx, sy, sz, want_saddles);
    k_list_back<<<pg, kBlock, 0, st>>>(T, L);
    ctx->launches += 3;
}

double key_to_double(unsigned long long k) {
    uint64_t b = (k & 0x8000000000000000ull) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
    double d;
    memcpy(&d, &b, 8);
    return d;
}

// min and max of a device field (exact)
dmtz_status device_minmax(dmtz_ctx *ctx, const double *a, i64 n, double &mn, double &mx) {
    unsigned long long init[2] = {~0ull, 0ull}, out[2];
    CK(cudaMemcpyAsync(ctx->counters + 8, init, sizeof(init), cudaMemcpyHostToDevice, ctx->stream));
    k_minmax<<<persistent_grid(), kBlock, 0, ctx->stream>>>(a, n, ctx->counters + 8, ctx->counters + 9);
    ctx->launches++;
    CK(cudaMemcpyAsync(out, ctx->counters + 8, sizeof(out), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    mn = key_to_double(out[0]);
    mx = key_to_double(out[1]);
    return DMTZ_OK;
}

RuleCtx rule_ctx(dmtz_ctx *ctx, const Grid &g, double bound, int edit_type) {
    RuleCtx c;
    c.g = g;
    c.P = view(ctx->P, ctx->f);
    c.Q = view(ctx->Q, ctx->g);
    c.f = ctx->f;
    c.gv = ctx->g;
    c.cnt = ctx->cnt;
    c.bound = bound;
    c.edit_type = edit_type;
    c.reqbits = ctx->reqbits;
    c.reqlist = ctx->reqlist;
    c.reqn = ctx->counters + 4;
    c.reqcap = g.V;
    c.err = ctx->errword;
    c.progress = ctx->counters + 7;
    return c;
}

// After a scan that left its counts in hc[0..3]: grow every overflowed list
// and scan again (same masks, so the same counts, which now fit).
dmtz_status fit_lists(dmtz_ctx *ctx, const Grid &g, int want_saddles, unsigned long long *hc) {
    bool over = false;
    for (int k = 0; k < 4; k++) {
        if ((i64)hc[k] <= ctx->capL[k]) continue;
        dmtz_status s = grow_list(ctx, g, k, (i64)hc[k]);
        if (s != DMTZ_OK) return s;
        over = true;
    }
    if (!over) return DMTZ_OK;
    scan_mismatch(ctx, g, ctx->Q.crit, ctx->P.crit, want_saddles);
    CK(cudaMemcpyAsync(hc, ctx->counters, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return DMTZ_OK;
}

CpLists cp_lists(const dmtz_ctx *ctx) {
    CpLists L;
    for (int k = 0; k < 4; k++) {
        L.l[k] = ctx->lists[k];
        L.cap[k] = ctx->capL[k];
    }
    L.n = ctx->counters;
    return L;
}

PathRec path_rec(const dmtz_ctx *ctx) {
    return PathRec{ctx->as_tet, ctx->as_cur, ctx->ds_edge, ctx->ds_vert, ctx->counters + 5, ctx->capAS, ctx->capDS};
}

// static data of the original ascending paths (after the original pairing),
// and record buffers sized by the original saddle counts (each original
// 2-saddle gives at most one ascending record, each 1-saddle at most one
// descending record)
// the rebuild buffers of the descending records, as large as the records
dmtz_status ensure_ds_tmp(dmtz_ctx *ctx) {
    const i64 need = std::max<i64>(ctx->capDS, 1);
    if (ctx->capDST >= need) return DMTZ_OK;
    cudaFree(ctx->ds_tmp_edge);
    cudaFree(ctx->ds_tmp_vert);
    ctx->ds_tmp_edge = ctx->ds_tmp_vert = nullptr;
    ctx->capDST = 0;
    CK(dalloc(&ctx->ds_tmp_edge, need));
    CK(dalloc(&ctx->ds_tmp_vert, need));
    ctx->capDST = need;
    return DMTZ_OK;
}

dmtz_status prep_paths(dmtz_ctx *ctx, const Grid &g) {
    cudaStream_t st = ctx->stream;
    dmtz_status s0;
    CK(cudaMemsetAsync(ctx->counters + 13, 0, 2 * sizeof(unsigned long long), st));
    k_count_saddles<<<persistent_grid(), kBlock, 0, st>>>(g.V, ctx->P.crit, ctx->counters + 13);
    unsigned long long n[2] = {0, 0};
    CK(cudaMemcpyAsync(n, ctx->counters + 13, sizeof(n), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if ((i64)n[0] > ctx->capDS) {
        cudaFree(ctx->ds_edge);
        cudaFree(ctx->ds_vert);
        ctx->ds_edge = ctx->ds_vert = nullptr;
        ctx->capDS = 0;
        CK(dalloc(&ctx->ds_edge, (i64)n[0]));
        CK(dalloc(&ctx->ds_vert, (i64)n[0]));
        ctx->capDS = (i64)n[0];
    }
    if ((i64)n[1] > ctx->capAS) {
        cudaFree(ctx->as_tet);
        cudaFree(ctx->as_cur);
        cudaFree(ctx->sad2);
        cudaFree(ctx->as_res);
        ctx->as_tet = ctx->as_cur = ctx->sad2 = ctx->as_res = nullptr;
        ctx->capAS = ctx->capSad2 = 0;
        CK(dalloc(&ctx->as_tet, (i64)n[1]));
        CK(dalloc(&ctx->as_cur, (i64)n[1]));
        CK(dalloc(&ctx->sad2, (i64)n[1]));
        CK(dalloc(&ctx->as_res, 2 * (i64)n[1]));
        ctx->capAS = ctx->capSad2 = (i64)n[1];
    }
    // buffers exist even when a count is 0 (kernels take their addresses)
    if (!ctx->ds_edge) {
        CK(dalloc(&ctx->ds_edge, 1));
        CK(dalloc(&ctx->ds_vert, 1));
    }
    if (!ctx->as_tet) {
        CK(dalloc(&ctx->as_tet, 1));
        CK(dalloc(&ctx->as_cur, 1));
        CK(dalloc(&ctx->sad2, 1));
        CK(dalloc(&ctx->as_res, 2));
    }
    if ((s0 = ensure_ds_tmp(ctx)) != DMTZ_OK) return s0;
    CK(cudaMemsetAsync(ctx->counters + 24, 0, 3 * sizeof(unsigned long long), st));
    // walk cache: every walk runs at the first detection
    const i64 nw = std::max<i64>(2 * (i64)n[1], 2);
    if (nw > ctx->capWB) {
        cudaFree(ctx->walk_box);
        ctx->walk_box = nullptr;
        ctx->capWB = 0;
        CK(dalloc(&ctx->walk_box, nw));
        ctx->capWB = nw;
    }
    ctx->ntx = (g.W + kTile - 1) / kTile;
    ctx->nty = (g.H + kTile - 1) / kTile;
    ctx->ntz = (g.D + kTile - 1) / kTile;
    const i64 nt = (i64)ctx->ntx * ctx->nty * ctx->ntz;
    if (nt > ctx->capTile) {
        cudaFree(ctx->tile_dirty);
        cudaFree(ctx->tile_sat);
        ctx->tile_dirty = nullptr;
        ctx->tile_sat = nullptr;
        ctx->capTile = 0;
        CK(dalloc(&ctx->tile_dirty, nt));
        CK(dalloc(&ctx->tile_sat, nt));
        ctx->capTile = nt;
    }
    CK(cudaMemsetAsync(ctx->walk_box, 0, sizeof(unsigned long long) * (size_t)nw, st));
    CK(cudaMemsetAsync(ctx->tile_dirty, 0, (size_t)nt, st));
    CK(cudaMemsetAsync(ctx->counters + 10, 0, sizeof(unsigned long long), st));
    k_path_succ<<<grid_for(g.V), kBlock, 0, st>>>(g, ctx->P.tcode, ctx->succ);
    k_crit_list<8, 12><<<persistent_grid(), kBlock, 0, st>>>(g, ctx->P.crit, ctx->sad2, ctx->capSad2,
                                                             ctx->counters + 10);
    if (ctx->strict_ds) {  // the whole-path descending checks walk from the 1-saddle list
        const i64 need = std::max<i64>((i64)n[0], 1);
        if (need > ctx->capSad1) {
            cudaFree(ctx->sad1);
            ctx->sad1 = nullptr;
            ctx->capSad1 = 0;
            CK(dalloc(&ctx->sad1, need));
            ctx->capSad1 = need;
        }
        CK(cudaMemsetAsync(ctx->counters + 28, 0, sizeof(unsigned long long), st));
        k_crit_list<1, 7><<<persistent_grid(), kBlock, 0, st>>>(g, ctx->P.crit, ctx->sad1, ctx->capSad1,
                                                                ctx->counters + 28);
        ctx->launches++;
    }
    ctx->launches += 3;
    CK(cudaGetLastError());
    return DMTZ_OK;
}

// separatrix detection (ascending and descending) into the path records
// geometry mode (conn = 0) or connectivity mode (conn = 1); no launch counting
// (also used while capturing the graph loop)
void launch_detect(dmtz_ctx *ctx, const Grid &g, const RuleCtx &rc, const PathRec &R, unsigned grid, int conn) {
    cudaStream_t st = ctx->stream;
    // the last detection's descending record count, for the incremental rebuild
    cudaMemcpyAsync(ctx->counters + 25, ctx->counters + 6, sizeof(unsigned long long), cudaMemcpyDeviceToDevice, st);
    cudaMemsetAsync(ctx->counters + 5, 0, 2 * sizeof(unsigned long long), st);
    if (conn) {
        k_conn_as<<<grid, kBlock, 0, st>>>(g, ctx->P.crit, ctx->Q.crit, ctx->P.tcode, ctx->Q.tcode, ctx->succ, R,
                                           g.T + 16, ctx->errword);
        k_conn_ds<<<grid, kBlock, 0, st>>>(rc, R, g.V + 16);
    } else {
        const int ntx = ctx->ntx, nty = ctx->nty, ntz = ctx->ntz;
        k_sat_x<<<grid_for((i64)nty * ntz), kBlock, 0, st>>>(ctx->tile_dirty, ctx->tile_sat, ntx, nty, ntz);
        k_sat_yz<<<grid_for((i64)ntx * ntz), kBlock, 0, st>>>(ctx->tile_sat, ntx, nty, ntz, 1);
        k_sat_yz<<<grid_for((i64)ntx * nty), kBlock, 0, st>>>(ctx->tile_sat, ntx, nty, ntz, 2);
        TileSat T;
        T.sat = ctx->tile_sat;
        T.ntx = ntx;
        T.nty = nty;
        T.ntz = ntz;
        cudaMemsetAsync(ctx->counters + 27, 0, sizeof(unsigned long long), st);  // the walks' ticket
        k_path_as_walk<<<grid, kBlock, 0, st>>>(g, ctx->sad2, ctx->counters + 10, ctx->P.tcode, ctx->Q.tcode,
                                                ctx->succ, ctx->as_res, g.T + 16, ctx->errword, ctx->walk_box, T,
                                                ctx->counters + 27);
        k_path_as_pick<<<grid, kBlock, 0, st>>>(g, ctx->sad2, ctx->counters + 10, ctx->as_res, R);
        if (ctx->strict_ds) {  // whole-path descending checks of every 1-saddle, into the records
            cudaMemsetAsync(ctx->counters + 29, 0, sizeof(unsigned long long), st);  // the walks' ticket
            k_ds_strict<<<grid, kBlock, 0, st>>>(rc, R, ctx->sad1, ctx->counters + 28, g.V + 16,
                                                 ctx->counters + 29);
            return;
        }
        cudaMemsetAsync(ctx->counters + 26, 0, sizeof(unsigned long long), st);
        k_ds_keep<<<grid, kBlock, 0, st>>>(g, R, ctx->counters + 25, ctx->counters + 24, ctx->ds_tmp_edge,
                                           ctx->ds_tmp_vert, ctx->counters + 26, ctx->capDST, T);
        k_ds_tiles<<<grid, kBlock, 0, st>>>(rc, ctx->counters + 24, ctx->ds_tmp_edge, ctx->ds_tmp_vert,
                                            ctx->counters + 26, ctx->capDST, T);
        k_ds_back<<<grid, kBlock, 0, st>>>(R, ctx->ds_tmp_edge, ctx->ds_tmp_vert, ctx->counters + 26,
                                           ctx->counters + 24);
    }
}
// kernels one detection launches
int detect_kernels(const dmtz_ctx *ctx, int conn) { return conn ? 2 : (ctx->strict_ds ? 6 : 8); }
void detect_paths(dmtz_ctx *ctx, const Grid &g, const RuleCtx &rc, const PathRec &R, unsigned grid, int conn = 0) {
    launch_detect(ctx, g, rc, R, grid, conn);
    ctx->launches += detect_kernels(ctx, conn);
}

// Wall records (preserve_connectors = 1) of the current decompressed gradient:
// every original 2-saddle searched by tiers (see wall_dfs).  Record arrays
// hold one entry per original 2-saddle; the deferred lists likewise.
dmtz_status ensure_walls(dmtz_ctx *ctx) {
    const i64 need = std::max<i64>(ctx->capSad2, 1);
    if (ctx->capWall >= need) return DMTZ_OK;
    cudaFree(ctx->wall_sad); cudaFree(ctx->wall_edge); cudaFree(ctx->wall_next[0]); cudaFree(ctx->wall_next[1]);
    ctx->wall_sad = ctx->wall_edge = ctx->wall_next[0] = ctx->wall_next[1] = nullptr;
    ctx->capWall = 0;
    CK(dalloc(&ctx->wall_sad, need));
    CK(dalloc(&ctx->wall_edge, need));
    CK(dalloc(&ctx->wall_next[0], need));
    CK(dalloc(&ctx->wall_next[1], need));
    ctx->capWall = need;
    return DMTZ_OK;
}
WallRec wall_rec(dmtz_ctx *ctx) {
    WallRec W;
    W.sad = ctx->wall_sad;
    W.edge = ctx->wall_edge;
    W.n = ctx->counters + 16;
    W.cap = ctx->capWall;
    return W;
}
unsigned persistent_grid();
dmtz_status detect_walls(dmtz_ctx *ctx, const Grid &g, const RuleCtx &rc, i64 &n_wall) {
    struct Tier {
        int stack_cap, cache_bits;
        long long pop_cap;
    };
    static const Tier tiers[3] = {{2048, 13, 1ll << 16}, {1 << 16, 18, 1ll << 22}, {1 << 21, 23, 1ll << 28}};
    const i64 budget = (i64)32 << 20;  // scratch entries (256 MB)
    cudaStream_t st = ctx->stream;
    dmtz_status s;
    if ((s = ensure_walls(ctx)) != DMTZ_OK) return s;
    const WallRec W = wall_rec(ctx);
    CK(cudaMemsetAsync(ctx->counters + 16, 0, 3 * sizeof(unsigned long long), st));
    k_wall_t1<<<persistent_grid(), kBlock, 0, st>>>(rc, ctx->sad2, ctx->counters + 10, ctx->capSad2, W,
                                                     ctx->wall_next[0], ctx->counters + 17, ctx->capWall);
    ctx->launches++;
    unsigned long long nd = 0;
    CK(cudaMemcpyAsync(&nd, ctx->counters + 17, sizeof(nd), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    int cur = 0;
    for (int t = 0; t < 3 && nd > 0; t++) {
        const Tier &T = tiers[t];
        const i64 per = (i64)T.stack_cap + ((i64)1 << T.cache_bits);
        const i64 chunk = std::max<i64>(1, std::min<i64>((i64)nd, budget / per));
        if (ctx->capWS < chunk * per) {
            cudaFree(ctx->wall_scratch);
            ctx->wall_scratch = nullptr;
            ctx->capWS = 0;
            CK(dalloc(&ctx->wall_scratch, chunk * per));
            ctx->capWS = chunk * per;
        }
        unsigned long long *nnext = ctx->counters + 17 + (cur ^ 1);
        CK(cudaMemsetAsync(nnext, 0, sizeof(unsigned long long), st));
        for (i64 first = 0; first < (i64)nd; first += chunk) {
            const i64 cnt = std::min<i64>(chunk, (i64)nd - first);
            k_wall_tn<<<grid_for(cnt), kBlock, 0, st>>>(rc, ctx->wall_next[cur], first, cnt, W, ctx->wall_next[cur ^ 1],
                                                        nnext, ctx->capWall, ctx->wall_scratch, T.stack_cap,
                                                        T.cache_bits, T.pop_cap);
            ctx->launches++;
        }
        CK(cudaMemcpyAsync(&nd, nnext, sizeof(nd), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        cur ^= 1;
    }
    if (nd > 0) return fail(ctx, DMTZ_ERR_TOO_LARGE, "a wall search outgrew its largest tier (2^21 stack entries)");
    unsigned long long nw = 0;
    CK(cudaMemcpyAsync(&nw, ctx->counters + 16, sizeof(nw), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    CK(cudaGetLastError());
    n_wall = (i64)nw;
    return DMTZ_OK;
}

unsigned persistent_grid() {
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return (unsigned)sms * 8;
}

dmtz_status check_dims(dmtz_ctx *ctx, int W, int H, int D, Grid &g) {
    if (!ctx) return DMTZ_ERR_ARG;
    if (W < 2 || H < 2 || D < 2) return fail(ctx, DMTZ_ERR_ARG, "dims must be >= 2");
    g = make_grid(W, H, D);
    if (!shape_fits(g, 0)) return fail(ctx, DMTZ_ERR_ARG, "dims exceed 16384 x 8192 x 4096");
    if (!shape_fits(g, ctx->tune_shape)) ctx->tune_shape = 0;
    return DMTZ_OK;
}

// NaN / Inf test of a device field (the reference assumes finite input)
dmtz_status check_finite(dmtz_ctx *ctx, const double *d, i64 n) {
    CK(cudaMemsetAsync(ctx->errword, 0, sizeof(int), ctx->stream));
    k_check_finite<<<persistent_grid(), kBlock, 0, ctx->stream>>>(d, n, ctx->errword);
    ctx->launches++;
    int bad = 0;
    CK(cudaMemcpyAsync(&bad, ctx->errword, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (bad) return fail(ctx, DMTZ_ERR_ARG, "input contains NaN or Inf");
    return DMTZ_OK;
}

dmtz_status upload(dmtz_ctx *ctx, double *dst, const double *src, i64 n, int on_device) {
    CK(cudaMemcpyAsync(dst, src, sizeof(double) * (size_t)n, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaMemsetAsync(ctx->errword, 0, sizeof(int), ctx->stream));
    k_check_finite<<<persistent_grid(), kBlock, 0, ctx->stream>>>(dst, n, ctx->errword);
    ctx->launches++;
    int bad = 0;
    CK(cudaMemcpyAsync(&bad, ctx->errword, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (bad) return fail(ctx, DMTZ_ERR_ARG, "input contains NaN or Inf");
    return DMTZ_OK;
}

}  // namespace

// =============================================================================
// C ABI
// =============================================================================
// Link components of every vertex (no counterpart in the reference, which
// classifies cells by the discrete gradient; this is the piecewise-linear
// reading of "min / max / saddle from the lower and upper link").  The
// Freudenthal triangulation is a flag complex, so the link of v has an edge
// between two stencil neighbours exactly when they are adjacent, and a
// triangle for every adjacent triple.  Lower (upper) link: the neighbours
// below (above) v in compare_vertices order (main_3d.cu:1043-1049).
namespace lnk {
__host__ __device__ constexpr uint32_t adj(int i) {
    uint32_t m = 0;
    for (int j = 0; j < 14; j++)
        if (j != i && cxt::cdir(cxt::TOPO_DIRS[i][0] - cxt::TOPO_DIRS[j][0], cxt::TOPO_DIRS[i][1] - cxt::TOPO_DIRS[j][1],
                                cxt::TOPO_DIRS[i][2] - cxt::TOPO_DIRS[j][2]) >= 0)
            m |= 1u << j;
    return m;
}
// the n-th adjacent triple i < j < k (packed i | j << 4 | k << 8), -1 past the end
__host__ __device__ constexpr int tri(int n) {
    for (int i = 0; i < 14; i++)
        for (int j = i + 1; j < 14; j++)
            for (int k = j + 1; k < 14; k++)
                if (((adj(i) >> j) & 1u) && ((adj(i) >> k) & 1u) && ((adj(j) >> k) & 1u) && n-- == 0)
                    return i | (j << 4) | (k << 8);
    return -1;
}
__host__ __device__ constexpr int ntri() {
    int n = 0;
    while (tri(n) >= 0) n++;
    return n;
}
// the neighbours reachable from `seed` inside m
__device__ __forceinline__ uint32_t grow(uint32_t seed, uint32_t m) {
    uint32_t comp = seed, prev = 0;
    while (comp != prev) {
        prev = comp;
        uint32_t nb = comp;
        DMTZ_FOR(14, I, {
            constexpr int i = decltype(I)::value;
            nb |= ((comp >> i) & 1u) ? adj(i) : 0u;
        });
        comp = nb & m;
    }
    return comp;
}
__device__ __forceinline__ int components(uint32_t m) {
    int c = 0;
    while (m) {
        m &= ~grow(m & (0u - m), m);
        c++;
    }
    return c;
}
// Euler characteristic of the link's full subcomplex on m
__device__ __forceinline__ int chi(uint32_t m) {
    int e2 = 0, t = 0;
    DMTZ_FOR(14, I, {
        constexpr int i = decltype(I)::value;
        e2 += ((m >> i) & 1u) ? __popc(adj(i) & m) : 0;
    });
    DMTZ_FOR(ntri(), N, {
        constexpr int p = tri(decltype(N)::value);
        t += (int)((m >> (p & 15)) & (m >> ((p >> 4) & 15)) & (m >> (p >> 8)) & 1u);
    });
    return __popc(m) - e2 / 2 + t;
}
}  // namespace lnk

__global__ void k_link_classes(Grid g, const double *data, uint8_t *out, unsigned long long *counts) {
    long long c[6] = {0, 0, 0, 0, 0, 0};
    for (i64 v = (i64)blockIdx.x * blockDim.x + threadIdx.x; v < g.V; v += (i64)gridDim.x * blockDim.x) {
        int x, y, z;
        decode_v(g, v, x, y, z);
        const uint64_t kv = okey(data[v]);
        uint32_t lo = 0, up = 0;
        DMTZ_FOR(14, I, {
            constexpr int i = decltype(I)::value;
            constexpr int dx = cxt::TOPO_DIRS[i][0], dy = cxt::TOPO_DIRS[i][1], dz = cxt::TOPO_DIRS[i][2];
            if (inb(g, x + dx, y + dy, z + dz)) {
                const uint64_t kn = okey(data[v + dx + dy * (i64)g.W + dz * g.WH]);
                const bool below = cxt::dir_up(i) ? (kn < kv) : (kn <= kv);
                lo |= below ? (1u << i) : 0u;
                up |= below ? 0u : (1u << i);
            }
        });
        const int cl = lnk::components(lo), cu = lnk::components(up);
        if (out) out[v] = (uint8_t)(cl | (cu << 4));
        c[0] += cl == 0;
        c[1] += cu == 0;
        c[2] += cl == 1 && cu == 1;
        c[3] += cl >= 2 ? cl - 1 : 0;
        c[4] += cu >= 2 ? cu - 1 : 0;
        c[5] += 1 - lnk::chi(lo);
    }
#pragma unroll
    for (int k = 0; k < 6; k++) {
        long long x = c[k];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) == 0 && x) atomicAdd(counts + k, (unsigned long long)x);
    }
}

// Separatrix agreement of two gradients (measurement and acceptance checks;
// no counterpart in the reference): per original 1-saddle edge, the descending
// labels of its two endpoints, and per original 2-saddle triangle, the
// ascending labels of its cofaces, in the original field (dP, aP) and in the
// decompressed one (dQ, aQ).  out: [0] endpoints compared, [1] equal, [2]
// cofaces compared, [3] equal, [4] anchor cells whose criticality differs.
__global__ void k_sep_agree(Grid g, const uint32_t *critP, const uint32_t *critQ, const i64 *dP, const i64 *dQ,
                            const i64 *aP, const i64 *aQ, unsigned long long *out) {
    unsigned long long c[5] = {0, 0, 0, 0, 0};
    for (i64 v = (i64)blockIdx.x * blockDim.x + threadIdx.x; v < g.V; v += (i64)gridDim.x * blockDim.x) {
        const uint32_t cp = critP[v];
        c[4] += __popc(cp ^ critQ[v]);
        const uint32_t m1 = (cp >> 1) & 0x7Fu, m2 = (cp >> 8) & 0xFFFu;
        if (!(m1 | m2)) continue;
        int x, y, z;
        decode_v(g, v, x, y, z);
        DMTZ_FOR(7, K, {
            constexpr int k = decltype(K)::value;
            constexpr int c0 = cxt::TOPO_EDGE_V[k][0], c1 = cxt::TOPO_EDGE_V[k][1];
            if ((m1 >> k) & 1u) {
                const i64 a = v + cxt::ccx(c0) + cxt::ccy(c0) * (i64)g.W + cxt::ccz(c0) * g.WH;
                const i64 b = v + cxt::ccx(c1) + cxt::ccy(c1) * (i64)g.W + cxt::ccz(c1) * g.WH;
                c[0] += 2;
                c[1] += (dP[a] == dQ[a]) + (dP[b] == dQ[b]);
            }
        });
        DMTZ_FOR(12, S, {
            constexpr int sl = decltype(S)::value;
            if ((m2 >> sl) & 1u) {
                DMTZ_FOR(cxt::TOPO_FACE_NCOF[sl], J, {
                    constexpr int j = decltype(J)::value;
                    constexpr int tx = cxt::TOPO_FACE_COF[sl][j][0], ty = cxt::TOPO_FACE_COF[sl][j][1],
                                  tz = cxt::TOPO_FACE_COF[sl][j][2], ts = cxt::TOPO_FACE_COF[sl][j][3];
                    if (cell_ok(g, x + tx, y + ty, z + tz, 1, 1, 1)) {
                        const i64 t = (v + tx + ty * (i64)g.W + tz * g.WH) * 6 + ts;
                        c[2] += 1;
                        c[3] += aP[t] == aQ[t];
                    }
                });
            }
        });
    }
#pragma unroll
    for (int k = 0; k < 5; k++) {
        unsigned long long x = c[k];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) == 0 && x) atomicAdd(out + k, x);
    }
}

extern "C" {

dmtz_status dmtz_ctx_create(dmtz_ctx **out, int device) {
    if (!out) return DMTZ_ERR_ARG;
    *out = nullptr;
    dmtz_ctx *ctx = new dmtz_ctx();
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete ctx;
        return DMTZ_ERR_CUDA;
    }
    *out = ctx;
    return DMTZ_OK;
}

void dmtz_ctx_destroy(dmtz_ctx *ctx) {
    if (!ctx) return;
    for (dmtz_ctx *w : ctx->pool) dmtz_ctx_destroy(w);
    ctx->pool.clear();
    cudaSetDevice(ctx->device);
    free_all(ctx);
    cudaFree(ctx->mm);
    cudaFree(ctx->bnd);
    cudaFree(ctx->loopctl);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    if (ctx->side_done) cudaEventDestroy(ctx->side_done);
    delete ctx;
}

const char *dmtz_last_error(const dmtz_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

dmtz_status dmtz_cell_counts(int W, int H, int D, int64_t out[4]) {
    if (W < 2 || H < 2 || D < 2 || !out) return DMTZ_ERR_ARG;
    Grid g = make_grid(W, H, D);
    out[0] = g.V; out[1] = g.E; out[2] = g.F; out[3] = g.T;
    return DMTZ_OK;
}

dmtz_status dmtz_extract(dmtz_ctx *ctx, int W, int H, int D, const double *data, int on_device, int32_t *PV,
                         int32_t *PE, int32_t *PF, int32_t *PT) {
    Grid g;
    dmtz_status s = check_dims(ctx, W, H, D, g);
    if (s != DMTZ_OK) return s;
    if (g.F >= INT32_MAX) return fail(ctx, DMTZ_ERR_ARG, "grid too large for 32-bit reference ids");
    CK(cudaSetDevice(ctx->device));
    if ((s = ensure(ctx, g)) != DMTZ_OK) return s;
    if ((s = upload(ctx, ctx->f, data, g.V, on_device)) != DMTZ_OK) return s;
    FieldState fs = view(ctx->P, ctx->f);
    run_pairing(ctx, g, fs, nullptr, 1);
    int32_t *d[4];
    const i64 n[4] = {g.V, g.E, g.F, g.T};
    for (int k = 0; k < 4; k++) CK(dalloc(&d[k], n[k]));
    k_export<<<grid_for(g.V), kBlock, 0, ctx->stream>>>(g, fs, d[0], d[1], d[2], d[3]);
    int32_t *h[4] = {PV, PE, PF, PT};
    for (int k = 0; k < 4; k++)
        CK(cudaMemcpyAsync(h[k], d[k], sizeof(int32_t) * (size_t)n[k], cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    for (int k = 0; k < 4; k++) cudaFree(d[k]);
    CK(cudaGetLastError());
    return DMTZ_OK;
}

// shared set-up of the two complexes for the parity entry points
static dmtz_status setup_pair(dmtz_ctx *ctx, const Grid &g, const double *orig, const double *decp) {
    dmtz_status s;
    if ((s = ensure(ctx, g)) != DMTZ_OK) return s;
    if ((s = upload(ctx, ctx->f, orig, g.V, 0)) != DMTZ_OK) return s;
    if ((s = upload(ctx, ctx->g, decp, g.V, 0)) != DMTZ_OK) return s;
    run_pairing(ctx, g, view(ctx->P, ctx->f), nullptr, 1);
    run_pairing(ctx, g, view(ctx->Q, ctx->g), ctx->P.crit, 1);
    CK(cudaGetLastError());
    unsigned long long hc[4];
    CK(cudaMemcpyAsync(hc, ctx->counters, sizeof(hc), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return fit_lists(ctx, g, 1, hc);
}

dmtz_status dmtz_mismatch(dmtz_ctx *ctx, int W, int H, int D, const double *orig, const double *decp,
                          int64_t counts[4], int32_t *lmin, int32_t *lsad, int32_t *l2sad, int32_t *lmax) {
    Grid g;
    dmtz_status s = check_dims(ctx, W, H, D, g);
    if (s != DMTZ_OK) return s;
    CK(cudaSetDevice(ctx->device));
    if ((s = setup_pair(ctx, g, orig, decp)) != DMTZ_OK) return s;
    unsigned long long hc[4];
    CK(cudaMemcpyAsync(hc, ctx->counters, sizeof(hc), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    int32_t *outs[4] = {lmin, lsad, l2sad, lmax};
    for (int k = 0; k < 4; k++) {
        counts[k] = (int64_t)hc[k];
        if (!outs[k] || !hc[k]) continue;
        std::vector<i64> tmp(hc[k]);
        CK(cudaMemcpy(tmp.data(), ctx->lists[k], sizeof(i64) * hc[k], cudaMemcpyDeviceToHost));
        std::sort(tmp.begin(), tmp.end());
        for (size_t i = 0; i < tmp.size(); i++) outs[k][i] = (int32_t)tmp[i];
    }
    return DMTZ_OK;
}

static void host_minmax(const double *f, i64 n, double &mn, double &mx) {
    mn = f[0]; mx = f[0];
    for (i64 i = 1; i < n; i++) {
        if (f[i] < mn) mn = f[i];
        if (f[i] > mx) mx = f[i];
    }
}

dmtz_status dmtz_fix_round(dmtz_ctx *ctx, int W, int H, int D, const double *orig, const double *decp,
                           const int32_t *edit_counter, double rel_eps, int preserve_saddles, int edit_type,
                           double *delta_out) {
    Grid g;
    dmtz_status s = check_dims(ctx, W, H, D, g);
    if (s != DMTZ_OK) return s;
    CK(cudaSetDevice(ctx->device));
    if ((s = setup_pair(ctx, g, orig, decp)) != DMTZ_OK) return s;
    double mn, mx;
    host_minmax(orig, g.V, mn, mx);
    const double range = mx - mn, bound = (mx - mn) * rel_eps;
    CK(cudaMemcpyAsync(ctx->cnt, edit_counter, sizeof(int) * (size_t)g.V, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemsetAsync(ctx->counters + 4, 0, sizeof(unsigned long long), ctx->stream));
    CK(cudaMemsetAsync(ctx->errword, 0, sizeof(int), ctx->stream));
    RuleCtx rc = rule_ctx(ctx, g, bound, edit_type);
    launch_fix_cp(rc, cp_lists(ctx), preserve_saddles, persistent_grid(), ctx->stream);
    double *dd = nullptr;
    CK(dalloc(&dd, g.V));
    const double sentinel = -2000.0 * range;
    std::vector<double> fill((size_t)g.V, sentinel);
    CK(cudaMemcpyAsync(dd, fill.data(), sizeof(double) * (size_t)g.V, cudaMemcpyHostToDevice, ctx->stream));
    // report the deltas the rules requested, without updating the field
    k_apply<<<persistent_grid(), kBlock, 0, ctx->stream>>>(rc, range, 0, 0, nullptr, dd);
    CK(cudaMemcpyAsync(delta_out, dd, sizeof(double) * (size_t)g.V, cudaMemcpyDeviceToHost, ctx->stream));
    int err = 0;
    CK(cudaMemcpyAsync(&err, ctx->errword, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    cudaFree(dd);
    CK(cudaGetLastError());
    if (err & ERR_OOB) return fail(ctx, DMTZ_ERR_OOB, "a fix rule indexed out of range");
    return DMTZ_OK;
}

static dmtz_status path_detect_impl(dmtz_ctx *ctx, int W, int H, int D, const double *orig, const double *decp,
                                    int conn, int64_t counts[2], int32_t *as_tet, int32_t *as_cur, int32_t *ds_edge,
                                    int32_t *ds_vert, int strict = 0) {
    Grid g;
    dmtz_status s = check_dims(ctx, W, H, D, g);
    if (s != DMTZ_OK) return s;
    ctx->strict_ds = strict && !conn;
    CK(cudaSetDevice(ctx->device));
    if ((s = setup_pair(ctx, g, orig, decp)) != DMTZ_OK) return s;
    CK(cudaMemsetAsync(ctx->errword, 0, sizeof(int), ctx->stream));
    RuleCtx rc = rule_ctx(ctx, g, 0.0, 0);
    if ((s = prep_paths(ctx, g)) != DMTZ_OK) return s;
    unsigned long long hc[2];
    int err = 0;
    for (int attempt = 0; attempt < 2; attempt++) {
        detect_paths(ctx, g, rc, path_rec(ctx), persistent_grid(), conn);
        CK(cudaMemcpyAsync(hc, ctx->counters + 5, sizeof(hc), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(&err, ctx->errword, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        // connectivity mode walks from the decompressed 2-saddles, which may
        // outnumber the original ones the records were sized for: grow, redo
        if ((i64)hc[0] <= ctx->capAS && (i64)hc[1] <= ctx->capDS) break;
        if ((i64)hc[0] > ctx->capAS) {
            cudaFree(ctx->as_tet);
            cudaFree(ctx->as_cur);
            ctx->as_tet = ctx->as_cur = nullptr;
            ctx->capAS = 0;
            CK(dalloc(&ctx->as_tet, (i64)hc[0]));
            CK(dalloc(&ctx->as_cur, (i64)hc[0]));
            ctx->capAS = (i64)hc[0];
        }
        if ((i64)hc[1] > ctx->capDS) {
            cudaFree(ctx->ds_edge);
            cudaFree(ctx->ds_vert);
            ctx->ds_edge = ctx->ds_vert = nullptr;
            ctx->capDS = 0;
            CK(dalloc(&ctx->ds_edge, (i64)hc[1]));
            CK(dalloc(&ctx->ds_vert, (i64)hc[1]));
            ctx->capDS = (i64)hc[1];
            if ((s = ensure_ds_tmp(ctx)) != DMTZ_OK) return s;
            // records past the old capacity were not kept: the next detection scans everything
            CK(cudaMemsetAsync(ctx->counters + 24, 0, sizeof(unsigned long long), ctx->stream));
        }
    }
    counts[0] = (int64_t)hc[0];
    counts[1] = (int64_t)hc[1];
    auto fetch = [&](i64 *da, i64 *db, unsigned long long n, int32_t *oa, int32_t *ob) -> dmtz_status {
        if (!n || !oa) return DMTZ_OK;
        std::vector<i64> a(n), b(n);
        CK(cudaMemcpy(a.data(), da, sizeof(i64) * n, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(b.data(), db, sizeof(i64) * n, cudaMemcpyDeviceToHost));
        std::vector<std::pair<i64, i64>> p(n);
        for (size_t i = 0; i < n; i++) p[i] = {a[i], b[i]};
        std::sort(p.begin(), p.end());
        for (size_t i = 0; i < n; i++) {
            oa[i] = (int32_t)p[i].first;
            if (ob) ob[i] = (int32_t)p[i].second;
        }
        return DMTZ_OK;
    };
    if ((s = fetch(ctx->as_tet, ctx->as_cur, hc[0], as_tet, as_cur)) != DMTZ_OK) return s;
    if ((s = fetch(ctx->ds_edge, ctx->ds_vert, hc[1], ds_edge, ds_vert)) != DMTZ_OK) return s;
    if (err & ERR_WALK) return fail(ctx, DMTZ_ERR_CYCLE, "a path walk exceeded its step cap");
    if (err & ERR_OOB) return fail(ctx, DMTZ_ERR_OOB, "a path rule indexed out of range");
    return DMTZ_OK;
}

dmtz_status dmtz_path_detect(dmtz_ctx *ctx, int W, int H, int D, const double *orig, const double *decp,
                             int64_t counts[2], int32_t *as_tet, int32_t *as_cur, int32_t *ds_edge,
                             int32_t *ds_vert) {
    return path_detect_impl(ctx, W, H, D, orig, decp, 0, counts, as_tet, as_cur, ds_edge, ds_vert);
}

dmtz_status dmtz_path_detect_strict(dmtz_ctx *ctx, int W, int H, int D, const double *orig, const double *decp,
                                    int64_t counts[2], int32_t *as_tet, int32_t *as_cur, int32_t *ds_edge,
                                    int32_t *ds_vert) {
    return path_detect_impl(ctx, W, H, D, orig, decp, 0, counts, as_tet, as_cur, ds_edge, ds_vert, 1);
}

dmtz_status dmtz_path_detect_connectivity(dmtz_ctx *ctx, int W, int H, int D, const double *orig,
                                          const double *decp, int64_t counts[2], int32_t *as_tet, int32_t *as_cur,
                                          int32_t *ds_edge, int32_t *ds_vert) {
    return path_detect_impl(ctx, W, H, D, orig, decp, 1, counts, as_tet, as_cur, ds_edge, ds_vert);
}

dmtz_status dmtz_wall_detect(dmtz_ctx *ctx, int W, int H, int D, const double *orig, const double *decp,
                             int64_t *count, int32_t *w_sad, int32_t *w_edge) {
    Grid g;
    dmtz_status s = check_dims(ctx, W, H, D, g);
    if (s != DMTZ_OK) return s;
    if (!count) return fail(ctx, DMTZ_ERR_ARG, "null count");
    CK(cudaSetDevice(ctx->device));
    if ((s = setup_pair(ctx, g, orig, decp)) != DMTZ_OK) return s;
    CK(cudaMemsetAsync(ctx->errword, 0, sizeof(int), ctx->stream));
    RuleCtx rc = rule_ctx(ctx, g, 0.0, 0);
    if ((s = prep_paths(ctx, g)) != DMTZ_OK) return s;
    i64 n = 0;
    if ((s = detect_walls(ctx, g, rc, n)) != DMTZ_OK) return s;
    *count = (int64_t)n;
    if (n > 0 && w_sad) {
        std::vector<i64> a(n), b(n);
        CK(cudaMemcpy(a.data(), ctx->wall_sad, sizeof(i64) * n, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(b.data(), ctx->wall_edge, sizeof(i64) * n, cudaMemcpyDeviceToHost));
        std::vector<std::pair<i64, i64>> p(n);
        for (i64 i = 0; i < n; i++) p[i] = {a[i], b[i]};
        std::sort(p.begin(), p.end());
        for (i64 i = 0; i < n; i++) {
            w_sad[i] = (int32_t)p[i].first;
            if (w_edge) w_edge[i] = (int32_t)p[i].second;
        }
    }
    int err = 0;
    CK(cudaMemcpy(&err, ctx->errword, sizeof(int), cudaMemcpyDeviceToHost));
    if (err & ERR_OOB) return fail(ctx, DMTZ_ERR_OOB, "a wall search indexed out of range");
    return DMTZ_OK;
}

// ----------------------------------------------------------------------------- graph-driven loop
// The host loop of main_3d.cu:6784-7149 as a state machine that runs on the
// device: a CUDA graph holds a WHILE node whose body switches on the state,
// runs that state's kernels, then lets one thread decide the next state and
// the loop condition from the device-side counters.  States:
//   CP     one critical-point round (fix rules, update, re-pair, mismatch)
//   PDF    path phase: detect separatrix records, fix, update, re-pair, mismatch
//   PCHECK detect separatrix records only (the reference's end-of-round check)
//   PFIX   path phase on the records PCHECK just made (the reference detects
//          them again at the start of its next outer iteration; same inputs,
//          same records)
namespace {
enum { LS_CP = 0, LS_PDF = 1, LS_PCHECK = 2, LS_PFIX = 3, LS_DONE = 4 };
struct LoopCtl {
    int state, pvp, converged, pad;
    long long rounds, max_rounds, outer, cp_rounds, path_rounds;
    long long cc[4];
    long long n_as, n_ds;
    long long runs[4];  // body executions per state
    long long cap[4];   // mismatch list capacities
    int overflow;       // a scan overflowed a list: stop, grow, scan again, resume at `state`
    int last;           // state of the last body run
    int break_stalls;   // stop when a round changed nothing (the host breaks the stall)
    int stalled;
};
}  // namespace

__global__ void k_set_switch(const LoopCtl *ctl, cudaGraphConditionalHandle h) {
    cudaGraphSetConditional(h, (unsigned)ctl->state);
}

__global__ void k_loop_ctl(LoopCtl *ctl, const unsigned long long *counters, cudaGraphConditionalHandle hwhile) {
    LoopCtl c = *ctl;
    const int st = c.state;
    c.runs[st]++;
    if (st != LS_PCHECK)
        for (int k = 0; k < 4; k++) c.cc[k] = (long long)counters[k];
    const bool cp_any = c.cc[0] > 0 || c.cc[1] > 0 || c.cc[2] > 0 || c.cc[3] > 0;
    int next;
    if (st == LS_CP) {
        c.rounds++;
        c.cp_rounds++;
        next = cp_any ? LS_CP : (c.pvp ? LS_PDF : LS_DONE);
    } else if (st == LS_PDF || st == LS_PFIX) {
        c.rounds++;
        c.path_rounds++;
        c.n_as = c.n_ds = 0;
        if (cp_any) {
            c.outer++;
            next = LS_CP;
        } else {
            next = LS_PCHECK;
        }
    } else {
        c.n_as = (long long)counters[5];
        c.n_ds = (long long)counters[6];
        if (c.n_as + c.n_ds > 0) {
            c.outer++;
            next = LS_PFIX;
        } else {
            next = LS_DONE;
        }
    }
    if (next != LS_DONE && c.rounds >= c.max_rounds) {
        c.converged = 0;
        next = LS_DONE;
    }
    c.last = st;
    if (next != LS_DONE && st != LS_PCHECK)
        for (int k = 0; k < 4; k++)
            if (c.cc[k] > c.cap[k]) c.overflow = 1;
    // counters[7]: set by the update when it changed something; a path round
    // counts only if its detection had records (counters[5], [6])
    if (c.break_stalls && next != LS_DONE && counters[7] == 0 &&
        (st == LS_CP || ((st == LS_PDF || st == LS_PFIX) && counters[5] + counters[6] > 0)))
        c.stalled = 1;
    c.state = next;
    *ctl = c;
    cudaGraphSetConditional(hwhile, (next != LS_DONE && !c.overflow && !c.stalled) ? 1u : 0u);
}

// ----------------------------------------------------------------------------- phase timers
namespace {
enum { PH_PAIR = 0, PH_FIXCP, PH_PATH, PH_FIXPATH, PH_APPLY, PH_SETUP, PH_N };
// event pairs recorded on the context's stream around each phase; summed once
// the stream has finished
struct PhaseTimer {
    cudaStream_t st;
    std::vector<cudaEvent_t> pool;
    std::vector<std::pair<int, size_t>> marks;  // phase, index of its first event
    size_t used = 0;
    cudaEvent_t next() {
        if (used == pool.size()) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            pool.push_back(e);
        }
        return pool[used++];
    }
    void begin(int ph) {
        marks.push_back({ph, used});
        cudaEventRecord(next(), st);
    }
    void end() { cudaEventRecord(next(), st); }
    void sum(double out[PH_N]) {
        for (int k = 0; k < PH_N; k++) out[k] = 0;
        for (auto &m : marks) {
            float t = 0;
            cudaEventElapsedTime(&t, pool[m.second], pool[m.second + 1]);
            out[m.first] += t;
        }
    }
    ~PhaseTimer() {
        for (auto e : pool) cudaEventDestroy(e);
    }
};
}  // namespace

// Build and run the graph-driven loop.  Returns the final LoopCtl in *out.
static dmtz_status run_graph_loop(dmtz_ctx *ctx, const Grid &g, const RuleCtx &rc, const CpLists &L,
                                  const PathRec &PR, const FieldState &Qs, double range, int ps, int pt, int conn,
                                  LoopCtl init, LoopCtl *out) {
    cudaStream_t st = ctx->stream;
    const unsigned pgrid = persistent_grid();
    if (!ctx->loopctl) CK(cudaMalloc(&ctx->loopctl, sizeof(LoopCtl)));
    LoopCtl *dctl = static_cast<LoopCtl *>(ctx->loopctl);
    CK(cudaMemcpyAsync(dctl, &init, sizeof(LoopCtl), cudaMemcpyHostToDevice, st));
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    dmtz_status res = DMTZ_OK;
    do {
        if (cudaGraphCreate(&graph, 0) != cudaSuccess) { res = DMTZ_ERR_CUDA; break; }
        cudaGraphConditionalHandle hwhile;
        if (cudaGraphConditionalHandleCreate(&hwhile, graph, 1, cudaGraphCondAssignDefault) != cudaSuccess) {
            res = DMTZ_ERR_CUDA;
            break;
        }
        cudaGraphNodeParams wp = {};
        wp.type = cudaGraphNodeTypeConditional;
        wp.conditional.handle = hwhile;
        wp.conditional.type = cudaGraphCondTypeWhile;
        wp.conditional.size = 1;
        cudaGraphNode_t wnode;
        if (cudaGraphAddNode(&wnode, graph, nullptr, nullptr, 0, &wp) != cudaSuccess) { res = DMTZ_ERR_CUDA; break; }
        cudaGraph_t body = wp.conditional.phGraph_out[0];
        cudaGraphConditionalHandle hsw;
        if (cudaGraphConditionalHandleCreate(&hsw, body, 0, 0) != cudaSuccess) { res = DMTZ_ERR_CUDA; break; }
        // body: set the switch from the state, switch over the four states, decide
        cudaGraphNode_t n_set, n_sw, n_ctl;
        {
            if (cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
                res = DMTZ_ERR_CUDA;
                break;
            }
            k_set_switch<<<1, 1, 0, st>>>(dctl, hsw);
            cudaGraph_t tmp;
            if (cudaStreamEndCapture(st, &tmp) != cudaSuccess) { res = DMTZ_ERR_CUDA; break; }
            size_t nn = 1;
            cudaGraphGetNodes(body, &n_set, &nn);
        }
        cudaGraphNodeParams sp = {};
        sp.type = cudaGraphNodeTypeConditional;
        sp.conditional.handle = hsw;
        sp.conditional.type = cudaGraphCondTypeSwitch;
        sp.conditional.size = 4;
        if (cudaGraphAddNode(&n_sw, body, &n_set, nullptr, 1, &sp) != cudaSuccess) { res = DMTZ_ERR_CUDA; break; }
        for (int state = 0; state < 4 && res == DMTZ_OK; state++) {
            cudaGraph_t child = sp.conditional.phGraph_out[state];
            if (cudaStreamBeginCaptureToGraph(st, child, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
                res = DMTZ_ERR_CUDA;
                break;
            }
            if (state == LS_PDF || state == LS_PCHECK) launch_detect(ctx, g, rc, PR, pgrid, conn);
            if (state != LS_PCHECK) {
                cudaMemsetAsync(ctx->counters + 4, 0, sizeof(unsigned long long), st);
                cudaMemsetAsync(ctx->counters + 7, 0, sizeof(unsigned long long), st);
                if (state == LS_CP) launch_fix_cp(rc, L, ps, pgrid, st);
                else k_fix_path<<<pgrid, kBlock, 0, st>>>(rc, PR);
                k_apply<<<pgrid, kBlock, 0, st>>>(rc, range, pt, 1, ctx->changed, nullptr);
                repair_dirty(ctx, g, Qs, ctx->P.crit, state == LS_CP ? (ps == 1) : 1);
            }
            cudaGraph_t tmp;
            if (cudaStreamEndCapture(st, &tmp) != cudaSuccess) res = DMTZ_ERR_CUDA;
        }
        if (res != DMTZ_OK) break;
        {
            if (cudaStreamBeginCaptureToGraph(st, body, &n_sw, nullptr, 1, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
                res = DMTZ_ERR_CUDA;
                break;
            }
            k_loop_ctl<<<1, 1, 0, st>>>(dctl, ctx->counters, hwhile);
            cudaGraph_t tmp;
            if (cudaStreamEndCapture(st, &tmp) != cudaSuccess) { res = DMTZ_ERR_CUDA; break; }
            (void)n_ctl;
        }
        if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) { res = DMTZ_ERR_CUDA; break; }
        if (cudaGraphLaunch(exec, st) != cudaSuccess) { res = DMTZ_ERR_CUDA; break; }
        if (cudaMemcpyAsync(out, dctl, sizeof(LoopCtl), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            res = DMTZ_ERR_CUDA;
    } while (0);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (res != DMTZ_OK) {
        cudaGetLastError();
        return fail(ctx, res, "building or running the loop graph failed");
    }
    return DMTZ_OK;
}

// ----------------------------------------------------------------------------- the correction loop
// features of (ctx->f, ctx->g) from the current gradients ctx->P / ctx->Q
static dmtz_status features_into(dmtz_ctx *ctx, const Grid &g, double bound, __nv_bfloat16 *feat, uint8_t *active) {
    if (g.V > ctx->capMM) {
        cudaFree(ctx->mm);
        ctx->mm = nullptr;
        ctx->capMM = 0;
        CK(dalloc(&ctx->mm, g.V));
        ctx->capMM = g.V;
    }
    cudaStream_t st = ctx->stream;
    const unsigned grid = persistent_grid();
    k_features<<<grid, kBlock, 0, st>>>(g, ctx->f, ctx->g, ctx->P.crit, ctx->Q.crit, bound, feat, ctx->mm);
    k_dilate<<<grid, kBlock, 0, st>>>(g, 0, ctx->mm, active);
    k_dilate<<<grid, kBlock, 0, st>>>(g, 1, active, ctx->mm);
    k_dilate<<<grid, kBlock, 0, st>>>(g, 2, ctx->mm, active);
    ctx->launches += 4;
    CK(cudaGetLastError());
    return DMTZ_OK;
}

// Learned warm start: features, network, proposal, then the gradient of the
// edited field (around the edits) and its mismatch lists again.
static dmtz_status learned_start(dmtz_ctx *ctx, dmtz_cnn *net, const Grid &g, double bound) {
    using namespace dmtz_cnn_impl;
    if (device_of(net) != ctx->device) return fail(ctx, DMTZ_ERR_ARG, "network and context on different devices");
    __nv_bfloat16 *feat;
    uint8_t *active;
    float *out;
    dmtz_status s = scratch(net, g.V, &feat, &active, &out);
    if (s != DMTZ_OK) return fail(ctx, s, "network: " + error_of(net));
    if ((s = features_into(ctx, g, bound, feat, active)) != DMTZ_OK) return s;
    s = forward_on(net, g.W, g.H, g.D, feat, out, 0, ctx->stream);
    if (s != DMTZ_OK) return fail(ctx, s, "network: " + error_of(net));
    CK(cudaMemsetAsync(ctx->counters + 4, 0, sizeof(unsigned long long), ctx->stream));
    k_propose<<<persistent_grid(), kBlock, 0, ctx->stream>>>(g.V, ctx->f, ctx->g, out, active, bound,
                                                              (double)min_drop_of(net) * bound, ctx->changed,
                                                              ctx->reqlist, ctx->counters + 4);
    ctx->launches += 5;
    // re-pair only the bricks within the passes' radii of the edited vertices
    // (the mismatch lists are rebuilt by a full scan: the loop has not started)
    repair_dirty(ctx, g, view(ctx->Q, ctx->g), ctx->P.crit, 1);
    CK(cudaMemsetAsync(ctx->counters + 4, 0, sizeof(unsigned long long), ctx->stream));
    CK(cudaGetLastError());
    return DMTZ_OK;
}

// a round made no progress: reset the values around the remaining mismatched
// cells (cp = 1) or separatrix records (cp = 0) to the original ones, re-pair
// there, and clear the request bits (see k_snap_cells)
static dmtz_status break_stall(dmtz_ctx *ctx, const Grid &g, const RuleCtx &rc, const PathRec &PR,
                               const FieldState &Qs, int cp, int want_saddles, int64_t nbreaks,
                               const WallRec *WR = nullptr) {
    cudaStream_t st = ctx->stream;
    const unsigned pgrid = persistent_grid();
    // the k-th break resets the box of half-width k around the seeds (the
    // seeds alone first), up to the whole grid, where g = f and every run ends
    const int radius = (int)std::min<int64_t>(nbreaks, std::max(g.W, std::max(g.H, g.D)));
    CK(cudaMemsetAsync(ctx->counters + 4, 0, sizeof(unsigned long long), st));
    if (cp) k_seed_cells<<<pgrid, kBlock, 0, st>>>(g, cp_lists(ctx), ctx->changed);
    else k_seed_paths<<<pgrid, kBlock, 0, st>>>(g, PR, ctx->changed);
    if (!cp && WR) {  // and the wall records' edges
        k_seed_walls<<<pgrid, kBlock, 0, st>>>(g, *WR, ctx->changed);
        ctx->launches++;
    }
    for (int axis = 0; axis < 3; axis++) {
        const int n = axis == 0 ? g.W : axis == 1 ? g.H : g.D;
        k_dilate_axis<<<grid_for(g.V / n), kBlock, 0, st>>>(g, ctx->changed, axis, std::min(radius, n));
    }
    k_snap_mask<<<pgrid, kBlock, 0, st>>>(rc, ctx->changed);
    repair_dirty(ctx, g, Qs, ctx->P.crit, want_saddles);
    k_clear_req<<<pgrid, kBlock, 0, st>>>(ctx->reqlist, ctx->counters + 4, g.V, ctx->reqbits);
    ctx->launches += 6;
    CK(cudaGetLastError());
    return DMTZ_OK;
}

static dmtz_status correct_impl(dmtz_ctx *ctx, dmtz_cnn *net, int W, int H, int D, const double *orig, double *decp,
                                int on_device, double rel_eps, const dmtz_opts *opts, dmtz_report *rep,
                                int32_t *edit_counter_out) {
    Grid g;
    dmtz_status s = check_dims(ctx, W, H, D, g);
    if (s != DMTZ_OK) return s;
    if (!opts) return fail(ctx, DMTZ_ERR_ARG, "null options");
    const int ps = opts->preserve_saddles, pvp = opts->preserve_vpath, pg = opts->preserve_geometry,
              filt = opts->filtration, pc = opts->preserve_connectors, pt = opts->preserve_type,
              et = opts->edit_type;
    // wall checks (preserve_connectors = 1) run in the separatrix phase; their
    // searches are sized on the host, so such runs use the host-driven loop
    const bool walls = pc == 1 && pvp == 1;
    const bool use_graph = opts->use_graph && !walls;
    const int conn = (pvp == 1 && pg == 0) ? 1 : 0;  // connectivity-mode separatrices
    if (!(rel_eps >= 0.0) || !std::isfinite(rel_eps)) return fail(ctx, DMTZ_ERR_ARG, "rel_eps must be finite and >= 0");
    const i64 max_rounds = opts->max_rounds > 0 ? opts->max_rounds : 100000;
    ctx->inc_scan = 0;  // full scans until the loop starts
    ctx->strict_ds = (opts->strict_separatrices && !conn) ? 1 : 0;
    CK(cudaSetDevice(ctx->device));
    if ((s = ensure(ctx, g)) != DMTZ_OK) return s;
    cudaStream_t st = ctx->stream;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    if ((s = upload(ctx, ctx->f, orig, g.V, on_device)) != DMTZ_OK) return s;
    // the decompressed field travels on a second stream while the original
    // field's gradient is computed; the work that reads it waits for it
    if (!ctx->side) {
        CK(cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&ctx->side_done, cudaEventDisableTiming));
    }
    CK(cudaMemcpyAsync(ctx->g, decp, sizeof(double) * (size_t)g.V,
                       on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, ctx->side));
    CK(cudaEventRecord(ctx->side_done, ctx->side));
    // range and bound exactly as the reference computes them (main_3d.cu:6303-6323)
    double mn, mx;
    ctx->launches = 0;
    PhaseTimer pt_{st};
    CK(cudaEventRecord(e0, st));
    pt_.begin(PH_SETUP);
    if ((s = device_minmax(ctx, ctx->f, g.V, mn, mx)) != DMTZ_OK) return s;
    const double bound = (mx - mn) * rel_eps;
    const double range = mx - mn;
    CK(cudaMemsetAsync(ctx->errword, 0, sizeof(int), st));
    CK(cudaMemsetAsync(ctx->changed, 0, (size_t)g.V, st));
    CK(cudaMemsetAsync(ctx->counters, 0, 8 * sizeof(unsigned long long), st));
    const FieldState Ps = view(ctx->P, ctx->f), Qs = view(ctx->Q, ctx->g);
    run_pairing(ctx, g, Ps, nullptr, 1);
    if (pvp == 1 && (s = prep_paths(ctx, g)) != DMTZ_OK) return s;
    CK(cudaStreamWaitEvent(st, ctx->side_done, 0));
    if ((s = check_finite(ctx, ctx->g, g.V)) != DMTZ_OK) return s;
    CK(cudaMemsetAsync(ctx->errword, 0, sizeof(int), st));
    if (filt == 1) {
        k_filter<<<grid_for(g.V), kBlock, 0, st>>>(g, ctx->P.crit, ctx->f, ctx->g, bound);
        ctx->launches++;
    }
    run_pairing(ctx, g, Qs, ctx->P.crit, 1);
    k_fill_i32<<<grid_for(g.V), kBlock, 0, st>>>(ctx->cnt, 1, g.V);
    ctx->launches++;
    pt_.end();
    unsigned long long hc[8];
    auto read_counts = [&]() -> dmtz_status {
        CK(cudaMemcpyAsync(hc, ctx->counters, sizeof(hc), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        return DMTZ_OK;
    };
    // counts after a mismatch scan; lists that overflowed grow and are rebuilt
    auto read_fit = [&](int want_saddles) -> dmtz_status {
        dmtz_status q = read_counts();
        return q != DMTZ_OK ? q : fit_lists(ctx, g, want_saddles, hc);
    };
    if ((s = read_fit(1)) != DMTZ_OK) return s;
    dmtz_report R;
    memset(&R, 0, sizeof(R));
    for (int k = 0; k < 4; k++) R.initial_mismatch[k] = (int64_t)hc[k];
    if (net) {
        pt_.begin(PH_SETUP);
        if ((s = learned_start(ctx, net, g, bound)) != DMTZ_OK) return s;
        pt_.end();
        if ((s = read_fit(1)) != DMTZ_OK) return s;
    }
    i64 cc[4] = {(i64)hc[0], (i64)hc[1], (i64)hc[2], (i64)hc[3]};
    i64 n_as = 1, n_ds = 1, n_wall = 1;
    // every scan of the loop asks for saddles when preserve_saddles = 1: the
    // repairs can then rebuild the lists from the re-paired bricks alone
    ctx->inc_scan = ps == 1 ? 1 : 0;
    i64 rounds = 0;
    int converged = 1;
    const unsigned pgrid = persistent_grid();
    RuleCtx rc = rule_ctx(ctx, g, bound, et);
    rc.range = range;
    const PathRec PR = path_rec(ctx);
    if (walls && (s = ensure_walls(ctx)) != DMTZ_OK) return s;
    const WallRec WR = wall_rec(ctx);
    auto cp_any = [&]() { return cc[0] > 0 || cc[1] > 0 || cc[2] > 0 || cc[3] > 0; };
    if (use_graph) {
        // same loop, decided on the device (see run_graph_loop)
        LoopCtl c;
        memset(&c, 0, sizeof(c));
        c.pvp = pvp;
        c.converged = 1;
        c.max_rounds = max_rounds;
        c.outer = 1;
        c.break_stalls = opts->break_stalls ? 1 : 0;
        for (int k = 0; k < 4; k++) c.cc[k] = cc[k];
        c.state = cp_any() ? LS_CP : (pvp ? LS_PDF : LS_DONE);
        LoopCtl fin = c;
        if (c.state != LS_DONE) {
            pt_.begin(PH_PAIR);
            LoopCtl cur = c;
            while (true) {
                for (int k = 0; k < 4; k++) cur.cap[k] = ctx->capL[k];
                if ((s = run_graph_loop(ctx, g, rc, cp_lists(ctx), PR, Qs, range, ps, pt, conn, cur, &fin)) != DMTZ_OK)
                    return s;
                if (!fin.overflow && !fin.stalled) break;
                // a scan outgrew a list: grow it, rebuild the lists and resume
                unsigned long long h4[4];
                for (int k = 0; k < 4; k++) h4[k] = (unsigned long long)fin.cc[k];
                if ((s = fit_lists(ctx, g, fin.last == LS_CP ? (ps == 1) : 1, h4)) != DMTZ_OK) return s;
                cur = fin;
                cur.overflow = 0;
                if (fin.stalled) {  // the round changed nothing: break the stall, then go on
                    const int cpst = fin.last == LS_CP;
                    if ((s = break_stall(ctx, g, rc, PR, Qs, cpst, cpst ? (ps == 1) : 1, R.stall_breaks)) != DMTZ_OK)
                        return s;
                    R.stall_breaks++;
                    if ((s = read_fit(cpst ? (ps == 1) : 1)) != DMTZ_OK) return s;
                    cur.stalled = 0;
                    for (int k = 0; k < 4; k++) cur.cc[k] = (long long)hc[k];
                    const bool any = hc[0] || hc[1] || hc[2] || hc[3];
                    if (cpst) {  // on with the critical-point loop, or to a separatrix round
                        cur.state = any ? LS_CP : (pvp ? LS_PDF : LS_DONE);
                    } else {  // a new outer iteration, or the separatrix re-check
                        cur.state = any ? LS_CP : LS_PCHECK;
                        if (any) cur.outer++;
                    }
                    if (cur.state == LS_DONE) {
                        fin = cur;
                        break;
                    }
                }
            }
            pt_.end();
            // kernels per body run: switch + control, plus each state's own
            const int64_t det = detect_kernels(ctx, conn);  // separatrix detection kernels
            // a fix round: fix + update, then the repair (dirty marks, compaction,
            // fresh and tile marks, six passes, the list rebuild)
            const int64_t rnd = 2 + 2 + (ctx->inc_scan ? 1 : 0) + (ctx->tile_dirty ? 1 : 0) + 6 + (ctx->inc_scan ? 3 : 1);
            const int64_t rnd_cp = rnd - 1 + (ps == 1 ? 5 : 3);  // the fix round's two forms (launch_fix_cp)
            ctx->launches += 2 * (fin.runs[0] + fin.runs[1] + fin.runs[2] + fin.runs[3]) + rnd_cp * fin.runs[LS_CP] +
                             (rnd + det) * fin.runs[LS_PDF] + det * fin.runs[LS_PCHECK] + rnd * fin.runs[LS_PFIX];
        }
        R.outer_iterations = fin.outer;
        R.cp_rounds = fin.cp_rounds;
        R.path_rounds = fin.path_rounds;
        for (int k = 0; k < 4; k++) cc[k] = fin.cc[k];
        n_as = fin.n_as;
        n_ds = fin.n_ds;
        n_wall = 0;
        converged = fin.converged;
    }
    // separatrix records of the last re-check, still valid while no round ran since
    bool paths_fresh = false;
    while (!use_graph && (n_as > 0 || n_ds > 0 || n_wall > 0 || cp_any())) {
        if (rounds >= max_rounds) {
            converged = 0;
            break;
        }
        R.outer_iterations++;
        while (cp_any()) {
            if (rounds >= max_rounds) break;
            rounds++;
            R.cp_rounds++;
            paths_fresh = false;
            CK(cudaMemsetAsync(ctx->counters + 4, 0, sizeof(unsigned long long), st));
            CK(cudaMemsetAsync(ctx->counters + 7, 0, sizeof(unsigned long long), st));
            pt_.begin(PH_FIXCP);
            const int nfix = launch_fix_cp(rc, cp_lists(ctx), ps, pgrid, st);
            pt_.end();
            pt_.begin(PH_APPLY);
            k_apply<<<pgrid, kBlock, 0, st>>>(rc, range, pt, 1, ctx->changed, nullptr);
            pt_.end();
            ctx->launches += nfix + 1;
            pt_.begin(PH_PAIR);
            repair_dirty(ctx, g, Qs, ctx->P.crit, ps == 1);
            pt_.end();
            if ((s = read_fit(ps == 1)) != DMTZ_OK) return s;
            if (opts->break_stalls && hc[7] == 0 && rounds < max_rounds && (hc[0] || hc[1] || hc[2] || hc[3])) {
                if ((s = break_stall(ctx, g, rc, PR, Qs, 1, ps == 1, R.stall_breaks)) != DMTZ_OK) return s;
                R.stall_breaks++;
                if ((s = read_fit(ps == 1)) != DMTZ_OK) return s;
            }
            for (int k = 0; k < 4; k++) cc[k] = (i64)hc[k];
        }
        if (rounds >= max_rounds) {
            converged = 0;
            break;
        }
        if (pvp == 0) break;
        // separatrix phase (main_3d.cu:6943-7148)
        rounds++;
        R.path_rounds++;
        if (!paths_fresh) {  // else the last re-check ran on this same state
            pt_.begin(PH_PATH);
            detect_paths(ctx, g, rc, PR, pgrid, conn);
            if (walls && (s = detect_walls(ctx, g, rc, n_wall)) != DMTZ_OK) return s;
            pt_.end();
        }
        const i64 walls_fixed = walls ? n_wall : 0;
        paths_fresh = false;
        CK(cudaMemsetAsync(ctx->counters + 4, 0, sizeof(unsigned long long), st));
        CK(cudaMemsetAsync(ctx->counters + 7, 0, sizeof(unsigned long long), st));
        pt_.begin(PH_FIXPATH);
        k_fix_path<<<pgrid, kBlock, 0, st>>>(rc, PR);
        if (walls_fixed > 0) {
            k_fix_wall<<<pgrid, kBlock, 0, st>>>(rc, WR);
            ctx->launches++;
        }
        pt_.end();
        pt_.begin(PH_APPLY);
        k_apply<<<pgrid, kBlock, 0, st>>>(rc, range, pt, 1, ctx->changed, nullptr);
        pt_.end();
        ctx->launches += 2;
        pt_.begin(PH_PAIR);
        repair_dirty(ctx, g, Qs, ctx->P.crit, 1);
        pt_.end();
        if ((s = read_fit(1)) != DMTZ_OK) return s;
        if (opts->break_stalls && hc[7] == 0 && rounds < max_rounds && hc[5] + hc[6] + walls_fixed > 0) {
            if ((s = break_stall(ctx, g, rc, PR, Qs, 0, 1, R.stall_breaks, walls_fixed > 0 ? &WR : nullptr)) !=
                DMTZ_OK)
                return s;
            R.stall_breaks++;
            if ((s = read_fit(1)) != DMTZ_OK) return s;
        }
        for (int k = 0; k < 4; k++) cc[k] = (i64)hc[k];
        n_as = n_ds = n_wall = 0;
        if (!cp_any()) {
            pt_.begin(PH_PATH);
            detect_paths(ctx, g, rc, PR, pgrid, conn);
            pt_.end();
            if ((s = read_counts()) != DMTZ_OK) return s;
            n_as = (i64)hc[5];
            n_ds = (i64)hc[6];
            if (walls && (s = detect_walls(ctx, g, rc, n_wall)) != DMTZ_OK) return s;
            paths_fresh = true;
        }
    }
    ctx->inc_scan = 0;
    CK(cudaEventRecord(e1, st));
    CK(cudaMemsetAsync(ctx->counters + 12, 0, sizeof(unsigned long long), st));
    k_count_u8<<<persistent_grid(), kBlock, 0, st>>>(ctx->changed, g.V, ctx->counters + 12);
    unsigned long long n_edited = 0;
    CK(cudaMemcpyAsync(&n_edited, ctx->counters + 12, sizeof(n_edited), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(decp, ctx->g, sizeof(double) * (size_t)g.V,
                       on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
    if (edit_counter_out)
        CK(cudaMemcpyAsync(edit_counter_out, ctx->cnt, sizeof(int) * (size_t)g.V, cudaMemcpyDeviceToHost, st));
    int err = 0;
    CK(cudaMemcpyAsync(&err, ctx->errword, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    CK(cudaGetLastError());
    for (int k = 0; k < 4; k++) R.final_mismatch[k] = cc[k];
    R.final_paths[0] = n_as;
    R.final_paths[1] = n_ds;
    R.final_walls = walls ? n_wall : 0;
    R.converged = converged;
    R.edited_vertices = (int64_t)n_edited;
    R.error_flags = err;
    R.seconds = ms * 1e-3;
    R.kernel_launches = ctx->launches;
    pt_.sum(R.phase_ms);
    if (rep) *rep = R;
    if (err & ERR_OOB) return fail(ctx, DMTZ_ERR_OOB, "a fix rule indexed out of range");
    if (err & ERR_WALK) return fail(ctx, DMTZ_ERR_CYCLE, "ascending path walk exceeded its step cap");
    if (!converged) return fail(ctx, DMTZ_ERR_NONCONVERGED, "round cap reached before the complexes agree");
    return DMTZ_OK;
}

dmtz_status dmtz_correct(dmtz_ctx *ctx, int W, int H, int D, const double *orig, double *decp, int on_device,
                         double rel_eps, const dmtz_opts *opts, dmtz_report *rep, int32_t *edit_counter_out) {
    return correct_impl(ctx, nullptr, W, H, D, orig, decp, on_device, rel_eps, opts, rep, edit_counter_out);
}

dmtz_status dmtz_correct_learned(dmtz_ctx *ctx, dmtz_cnn *net, int W, int H, int D, const double *orig,
                                 double *decp, int on_device, double rel_eps, const dmtz_opts *opts,
                                 dmtz_report *rep, int32_t *edit_counter_out) {
    if (!net) return fail(ctx, DMTZ_ERR_ARG, "null network");
    return correct_impl(ctx, net, W, H, D, orig, decp, on_device, rel_eps, opts, rep, edit_counter_out);
}

dmtz_status dmtz_quantize(dmtz_ctx *ctx, int W, int H, int D, const double *orig, double *decp, int on_device,
                          double rel_eps, double noise_frac, uint64_t seed) {
    Grid g;
    dmtz_status s = check_dims(ctx, W, H, D, g);
    if (s != DMTZ_OK) return s;
    if (!orig || !decp) return fail(ctx, DMTZ_ERR_ARG, "null field");
    if (!(rel_eps >= 0.0) || !std::isfinite(rel_eps) || !(noise_frac >= 0.0 && noise_frac <= 1.0))
        return fail(ctx, DMTZ_ERR_ARG, "rel_eps must be finite and >= 0, noise_frac in [0, 1]");
    CK(cudaSetDevice(ctx->device));
    if (!ctx->counters) {
        CK(dalloc(&ctx->counters, 32));
        CK(dalloc(&ctx->errword, 1));
    }
    cudaStream_t st = ctx->stream;
    const double *fd = orig;
    double *gd = decp;
    double *tmp = nullptr;
    if (!on_device) {  // staging buffers for host fields
        CK(dalloc(&tmp, 2 * g.V));
        CK(cudaMemcpyAsync(tmp, orig, sizeof(double) * (size_t)g.V, cudaMemcpyHostToDevice, st));
        fd = tmp;
        gd = tmp + g.V;
    }
    CK(cudaMemsetAsync(ctx->errword, 0, sizeof(int), st));
    k_check_finite<<<persistent_grid(), kBlock, 0, st>>>(fd, g.V, ctx->errword);
    int bad = 0;
    CK(cudaMemcpyAsync(&bad, ctx->errword, sizeof(int), cudaMemcpyDeviceToHost, st));
    double mn, mx;
    if ((s = device_minmax(ctx, fd, g.V, mn, mx)) != DMTZ_OK) {
        cudaFree(tmp);
        return s;
    }
    if (bad) {
        cudaFree(tmp);
        return fail(ctx, DMTZ_ERR_ARG, "input contains NaN or Inf");
    }
    k_quantize<<<persistent_grid(), kBlock, 0, st>>>(g.V, fd, gd, mn, (mx - mn) * rel_eps, noise_frac, seed);
    if (!on_device) CK(cudaMemcpyAsync(decp, gd, sizeof(double) * (size_t)g.V, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    cudaFree(tmp);
    CK(cudaGetLastError());
    return DMTZ_OK;
}

dmtz_status dmtz_features(dmtz_ctx *ctx, int W, int H, int D, const double *orig, const double *decp, int on_device,
                          double rel_eps, void *feat, uint8_t *active) {
    Grid g;
    dmtz_status s = check_dims(ctx, W, H, D, g);
    if (s != DMTZ_OK) return s;
    if (!feat || !active || ((uintptr_t)feat & 15)) return fail(ctx, DMTZ_ERR_ARG, "feat must be 16-byte aligned");
    if (!(rel_eps >= 0.0) || !std::isfinite(rel_eps)) return fail(ctx, DMTZ_ERR_ARG, "rel_eps must be finite and >= 0");
    CK(cudaSetDevice(ctx->device));
    if ((s = ensure(ctx, g)) != DMTZ_OK) return s;
    if ((s = upload(ctx, ctx->f, orig, g.V, on_device)) != DMTZ_OK) return s;
    if ((s = upload(ctx, ctx->g, decp, g.V, on_device)) != DMTZ_OK) return s;
    double mn, mx;
    if ((s = device_minmax(ctx, ctx->f, g.V, mn, mx)) != DMTZ_OK) return s;
    run_pairing(ctx, g, view(ctx->P, ctx->f), nullptr, 1);
    run_pairing(ctx, g, view(ctx->Q, ctx->g), nullptr, 1);
    if ((s = features_into(ctx, g, (mx - mn) * rel_eps, static_cast<__nv_bfloat16 *>(feat), active)) != DMTZ_OK)
        return s;
    CK(cudaStreamSynchronize(ctx->stream));
    return DMTZ_OK;
}

// pointer jumping to a fixed point; false if it does not settle within the cap
static dmtz_status jump_to_roots(dmtz_ctx *ctx, i64 *lab, i64 n) {
    for (int round = 0; round < 64; round++) {
        CK(cudaMemsetAsync(ctx->errword, 0, sizeof(int), ctx->stream));
        k_jump<<<persistent_grid(), kBlock, 0, ctx->stream>>>(lab, n, ctx->errword);
        int changed = 0;
        CK(cudaMemcpyAsync(&changed, ctx->errword, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        if (!changed) return DMTZ_OK;
    }
    return fail(ctx, DMTZ_ERR_CYCLE, "manifold labels did not settle (cycle in the gradient paths)");
}

dmtz_status dmtz_labels(dmtz_ctx *ctx, int W, int H, int D, const double *data, int on_device, int32_t *desc,
                        int32_t *asc) {
    Grid g;
    dmtz_status s = check_dims(ctx, W, H, D, g);
    if (s != DMTZ_OK) return s;
    if (g.F >= INT32_MAX) return fail(ctx, DMTZ_ERR_ARG, "grid too large for 32-bit reference ids");
    CK(cudaSetDevice(ctx->device));
    if ((s = ensure(ctx, g)) != DMTZ_OK) return s;
    if ((s = upload(ctx, ctx->f, data, g.V, on_device)) != DMTZ_OK) return s;
    run_pairing(ctx, g, view(ctx->P, ctx->f), nullptr, 1);
    k_path_succ<<<grid_for(g.V), kBlock, 0, ctx->stream>>>(g, ctx->P.tcode, ctx->succ);
    i64 *dl = nullptr, *al = nullptr;
    int32_t *dout = nullptr, *aout = nullptr;
    CK(dalloc(&dl, g.V));
    CK(dalloc(&al, 6 * g.V));
    CK(dalloc(&dout, g.V));
    CK(dalloc(&aout, g.T));
    const unsigned pg = persistent_grid();
    k_desc_init<<<pg, kBlock, 0, ctx->stream>>>(g, ctx->P.pv, dl);
    k_asc_init<<<pg, kBlock, 0, ctx->stream>>>(g, ctx->P.tcode, ctx->succ, al);
    if ((s = jump_to_roots(ctx, dl, g.V)) == DMTZ_OK) s = jump_to_roots(ctx, al, 6 * g.V);
    if (s == DMTZ_OK) {
        k_desc_out<<<pg, kBlock, 0, ctx->stream>>>(g, dl, dout);
        k_asc_out<<<pg, kBlock, 0, ctx->stream>>>(g, al, aout);
        CK(cudaMemcpyAsync(desc, dout, sizeof(int32_t) * (size_t)g.V, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(asc, aout, sizeof(int32_t) * (size_t)g.T, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    cudaFree(dl);
    cudaFree(al);
    cudaFree(dout);
    cudaFree(aout);
    CK(cudaGetLastError());
    return s;
}

dmtz_status dmtz_separatrix_agreement(dmtz_ctx *ctx, int W, int H, int D, const double *orig, const double *decp,
                                      int on_device, int64_t out[5]) {
    Grid g;
    dmtz_status s = check_dims(ctx, W, H, D, g);
    if (s != DMTZ_OK) return s;
    if (!out) return fail(ctx, DMTZ_ERR_ARG, "null output");
    CK(cudaSetDevice(ctx->device));
    if ((s = ensure(ctx, g)) != DMTZ_OK) return s;
    if ((s = upload(ctx, ctx->f, orig, g.V, on_device)) != DMTZ_OK) return s;
    if ((s = upload(ctx, ctx->g, decp, g.V, on_device)) != DMTZ_OK) return s;
    cudaStream_t st = ctx->stream;
    run_pairing(ctx, g, view(ctx->P, ctx->f), nullptr, 1);
    run_pairing(ctx, g, view(ctx->Q, ctx->g), nullptr, 1);
    i64 *dP = nullptr, *dQ = nullptr, *aP = nullptr, *aQ = nullptr;
    uint8_t *succQ = nullptr;
    unsigned long long *cnt = nullptr;
    auto release = [&]() {
        cudaFree(dP); cudaFree(dQ); cudaFree(aP); cudaFree(aQ); cudaFree(succQ); cudaFree(cnt);
    };
    if (dalloc(&dP, g.V) != cudaSuccess || dalloc(&dQ, g.V) != cudaSuccess || dalloc(&aP, 6 * g.V) != cudaSuccess ||
        dalloc(&aQ, 6 * g.V) != cudaSuccess || dalloc(&succQ, 8 * g.V) != cudaSuccess || dalloc(&cnt, 5) != cudaSuccess) {
        release();
        return fail(ctx, DMTZ_ERR_CUDA, "cannot allocate label buffers");
    }
    const unsigned pg = persistent_grid();
    k_path_succ<<<grid_for(g.V), kBlock, 0, st>>>(g, ctx->P.tcode, ctx->succ);
    k_path_succ<<<grid_for(g.V), kBlock, 0, st>>>(g, ctx->Q.tcode, succQ);
    k_desc_init<<<pg, kBlock, 0, st>>>(g, ctx->P.pv, dP);
    k_desc_init<<<pg, kBlock, 0, st>>>(g, ctx->Q.pv, dQ);
    k_asc_init<<<pg, kBlock, 0, st>>>(g, ctx->P.tcode, ctx->succ, aP);
    k_asc_init<<<pg, kBlock, 0, st>>>(g, ctx->Q.tcode, succQ, aQ);
    s = jump_to_roots(ctx, dP, g.V);
    if (s == DMTZ_OK) s = jump_to_roots(ctx, dQ, g.V);
    if (s == DMTZ_OK) s = jump_to_roots(ctx, aP, 6 * g.V);
    if (s == DMTZ_OK) s = jump_to_roots(ctx, aQ, 6 * g.V);
    if (s == DMTZ_OK) {
        unsigned long long h[5];
        if (cudaMemsetAsync(cnt, 0, 5 * sizeof(unsigned long long), st) != cudaSuccess) s = DMTZ_ERR_CUDA;
        k_sep_agree<<<pg, kBlock, 0, st>>>(g, ctx->P.crit, ctx->Q.crit, dP, dQ, aP, aQ, cnt);
        if (s == DMTZ_OK && (cudaMemcpyAsync(h, cnt, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                             cudaStreamSynchronize(st) != cudaSuccess))
            s = fail(ctx, DMTZ_ERR_CUDA, "label comparison failed");
        if (s == DMTZ_OK)
            for (int k = 0; k < 5; k++) out[k] = (int64_t)h[k];
    }
    release();
    CK(cudaGetLastError());
    return s;
}

dmtz_status dmtz_link_classes(dmtz_ctx *ctx, int W, int H, int D, const double *data, int on_device, uint8_t *out,
                              int64_t counts[6]) {
    Grid g;
    dmtz_status s = check_dims(ctx, W, H, D, g);
    if (s != DMTZ_OK) return s;
    if (!counts) return fail(ctx, DMTZ_ERR_ARG, "null counts");
    CK(cudaSetDevice(ctx->device));
    if ((s = ensure(ctx, g)) != DMTZ_OK) return s;
    if ((s = upload(ctx, ctx->f, data, g.V, on_device)) != DMTZ_OK) return s;
    cudaStream_t st = ctx->stream;
    uint8_t *dout = nullptr;
    unsigned long long *cnt = nullptr;
    if ((out && dalloc(&dout, g.V) != cudaSuccess) || dalloc(&cnt, 6) != cudaSuccess) {
        cudaFree(dout);
        return fail(ctx, DMTZ_ERR_CUDA, "cannot allocate link buffers");
    }
    unsigned long long h[6];
    cudaError_t e = cudaMemsetAsync(cnt, 0, sizeof(h), st);
    k_link_classes<<<persistent_grid(), kBlock, 0, st>>>(g, ctx->f, dout, cnt);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, cnt, sizeof(h), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && out) e = cudaMemcpyAsync(out, dout, (size_t)g.V, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(dout);
    cudaFree(cnt);
    if (e != cudaSuccess) return fail(ctx, DMTZ_ERR_CUDA, cudaGetErrorString(e));
    for (int k = 0; k < 6; k++) counts[k] = (int64_t)h[k];
    CK(cudaGetLastError());
    return DMTZ_OK;
}

dmtz_status dmtz_device_name(const dmtz_ctx *ctx, char *buf, int len) {
    if (!ctx || !buf || len < 1) return DMTZ_ERR_ARG;
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, ctx->device) != cudaSuccess) return DMTZ_ERR_CUDA;
    snprintf(buf, (size_t)len, "%s", p.name);
    return DMTZ_OK;
}

dmtz_status dmtz_set_tuning(dmtz_ctx *ctx, int shape, int blocks_per_sm) {
    if (!ctx || shape < 0 || shape >= DMTZ_NSHAPES || blocks_per_sm < 1 || blocks_per_sm > 64) return DMTZ_ERR_ARG;
    ctx->tune_shape = shape;
    ctx->tune_bps = blocks_per_sm;
    return DMTZ_OK;
}

dmtz_status dmtz_set_list_reserve(dmtz_ctx *ctx, double fraction, int64_t min_entries) {
    if (!ctx || !(fraction >= 0.0 && fraction <= 1.0) || min_entries < 1) return DMTZ_ERR_ARG;
    ctx->list_frac = fraction;
    ctx->list_min = min_entries;
    cudaSetDevice(ctx->device);
    for (int k = 0; k < 4; k++) {  // reallocated with the new reserve by the next call
        cudaFree(ctx->lists[k]);
        cudaFree(ctx->list_tmp[k]);
        ctx->lists[k] = ctx->list_tmp[k] = nullptr;
        ctx->capL[k] = 0;
    }
    return DMTZ_OK;
}

dmtz_status dmtz_get_tuning(const dmtz_ctx *ctx, int *shape, int *blocks_per_sm) {
    if (!ctx) return DMTZ_ERR_ARG;
    if (shape) *shape = ctx->tune_shape;
    if (blocks_per_sm) *blocks_per_sm = ctx->tune_bps;
    return DMTZ_OK;
}

dmtz_status dmtz_autotune(dmtz_ctx *ctx, int W, int H, int D, const double *orig, const double *decp, int on_device,
                          int best[2], double *best_ms) {
    Grid g;
    dmtz_status s = check_dims(ctx, W, H, D, g);
    if (s != DMTZ_OK) return s;
    CK(cudaSetDevice(ctx->device));
    if ((s = ensure(ctx, g)) != DMTZ_OK) return s;
    if ((s = upload(ctx, ctx->f, orig, g.V, on_device)) != DMTZ_OK) return s;
    if ((s = upload(ctx, ctx->g, decp, g.V, on_device)) != DMTZ_OK) return s;
    cudaStream_t st = ctx->stream;
    const FieldState Ps = view(ctx->P, ctx->f), Qs = view(ctx->Q, ctx->g);
    run_pairing(ctx, g, Ps, nullptr, 1);
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    static const int bps_opts[4] = {8, 16, 32, 64};
    double best_t = 1e30;
    int bs = 0, bb = 32;
    for (int sh = 0; sh < DMTZ_NSHAPES; sh++) {
        if (!shape_fits(g, sh)) continue;
        for (int bi = 0; bi < 4; bi++) {
            ctx->tune_shape = sh;
            ctx->tune_bps = bps_opts[bi];
            run_pairing(ctx, g, Qs, nullptr, 1);  // warm
            float t_min = 1e30f;
            for (int r = 0; r < 3; r++) {
                CK(cudaEventRecord(e0, st));
                run_pairing(ctx, g, Qs, nullptr, 1);
                CK(cudaEventRecord(e1, st));
                CK(cudaEventSynchronize(e1));
                float t = 0;
                cudaEventElapsedTime(&t, e0, e1);
                t_min = std::min(t_min, t);
            }
            if (t_min < best_t) {
                best_t = t_min;
                bs = sh;
                bb = bps_opts[bi];
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx->tune_shape = bs;
    ctx->tune_bps = bb;
    if (best) {
        best[0] = bs;
        best[1] = bb;
    }
    if (best_ms) *best_ms = best_t;
    CK(cudaGetLastError());
    return DMTZ_OK;
}

dmtz_status dmtz_correct_batch(dmtz_ctx *ctx, int n, const dmtz_instance *inst, const dmtz_opts *opts,
                               dmtz_report *reports, dmtz_status *status, int workers) {
    if (!ctx || n < 0 || (n > 0 && (!inst || !opts))) return DMTZ_ERR_ARG;
    if (workers < 1) workers = 8;
    workers = std::min(workers, std::max(n, 1));
    while ((int)ctx->pool.size() < workers) {
        dmtz_ctx *w = nullptr;
        const dmtz_status cs = dmtz_ctx_create(&w, ctx->device);
        if (cs != DMTZ_OK) return fail(ctx, cs, "cannot create a worker context");
        ctx->pool.push_back(w);
    }
    // every worker's buffers are sized once for the largest extents of the
    // batch: a reallocation in the middle would free device memory, and
    // cudaFree waits for the whole device, i.e. for the other workers
    int mW = 2, mH = 2, mD = 2;
    for (int i = 0; i < n; i++) {
        mW = std::max(mW, inst[i].W);
        mH = std::max(mH, inst[i].H);
        mD = std::max(mD, inst[i].D);
    }
    Grid gmax;
    if (n > 0 && check_dims(ctx, mW, mH, mD, gmax) == DMTZ_OK) {
        for (int k = 0; k < workers; k++) {
            dmtz_ctx *w = ctx->pool[k];
            w->list_frac = ctx->list_frac;
            w->list_min = ctx->list_min;
            cudaSetDevice(w->device);
            const dmtz_status es = ensure(w, gmax);
            if (es != DMTZ_OK) return fail(ctx, es, "cannot size worker buffers: " + w->err);
        }
    }
    std::atomic<int> next(0);
    std::vector<dmtz_status> st((size_t)n, DMTZ_OK);
    auto work = [&](dmtz_ctx *w) {
        w->tune_shape = ctx->tune_shape;
        w->tune_bps = ctx->tune_bps;
        w->list_frac = ctx->list_frac;
        w->list_min = ctx->list_min;
        std::vector<double> fo, go;
        for (int i = next++; i < n; i = next++) {
            const dmtz_instance &I = inst[i];
            const size_t V = (size_t)std::max(I.W, 0) * (size_t)std::max(I.H, 0) * (size_t)std::max(I.D, 0);
            if (!I.orig || !I.decp || !I.out || V == 0 || (I.dtype != DMTZ_F64 && I.dtype != DMTZ_F32)) {
                st[i] = DMTZ_ERR_ARG;
                continue;
            }
            const double *f64 = (const double *)I.orig;
            if (I.dtype == DMTZ_F32) {  // float32 widens exactly; the correction runs in float64
                fo.resize(V);
                const float *a = (const float *)I.orig, *b = (const float *)I.decp;
                for (size_t k = 0; k < V; k++) {
                    fo[k] = a[k];
                    I.out[k] = b[k];
                }
                f64 = fo.data();
            } else {
                memcpy(I.out, I.decp, V * sizeof(double));
            }
            dmtz_report r;
            st[i] = dmtz_correct(w, I.W, I.H, I.D, f64, I.out, 0, I.rel_eps, opts, &r, nullptr);
            if (reports) reports[i] = r;
        }
    };
    std::vector<std::thread> th;
    for (int k = 0; k < workers; k++) th.emplace_back(work, ctx->pool[k]);
    for (auto &t : th) t.join();
    dmtz_status res = DMTZ_OK;
    for (int i = 0; i < n; i++) {
        if (status) status[i] = st[i];
        if (st[i] != DMTZ_OK && res == DMTZ_OK) {
            res = st[i];
            ctx->err = "instance " + std::to_string(i) + " failed with status " + std::to_string((int)st[i]);
        }
    }
    return res;
}

dmtz_status dmtz_profile_sweep(dmtz_ctx *ctx, int W, int H, int D, const double *orig, const double *decp,
                               int on_device, int reps, double ms[7]) {
    Grid g;
    dmtz_status s = check_dims(ctx, W, H, D, g);
    if (s != DMTZ_OK) return s;
    if (reps < 1) return fail(ctx, DMTZ_ERR_ARG, "reps must be >= 1");
    CK(cudaSetDevice(ctx->device));
    if ((s = ensure(ctx, g)) != DMTZ_OK) return s;
    if ((s = upload(ctx, ctx->f, orig, g.V, on_device)) != DMTZ_OK) return s;
    if ((s = upload(ctx, ctx->g, decp, g.V, on_device)) != DMTZ_OK) return s;
    cudaStream_t st = ctx->stream;
    const FieldState Ps = view(ctx->P, ctx->f), Qs = view(ctx->Q, ctx->g);
    run_pairing(ctx, g, Ps, nullptr, 1);
    run_pairing(ctx, g, Qs, ctx->P.crit, 1);  // warm-up
    cudaEvent_t ev[7];
    for (auto &e : ev) CK(cudaEventCreate(&e));
    double acc[6] = {0, 0, 0, 0, 0, 0};
    float total = 0;
    i64 nb;
    const BrickList bl = all_bricks(g, ctx->tune_shape, nb);
    const unsigned gr = sweep_grid(ctx, nb);
    // as a full sweep runs them: each pass's brick kernel, then its surface anchors
    const int sk = surface_list(ctx, g) ? 1 : 0;
    const i64 *bd = ctx->bnd;
    const i64 nbd = sk ? ctx->bnd_n : 0;
    for (int r = 0; r < reps; r++) {
        CK(cudaEventRecord(ev[0], st));
        launch_pass<PASS_VERTEX>(g, Qs, bl, gr, st, sk);
        launch_bnd<PASS_VERTEX>(g, Qs, bd, nbd, st);
        CK(cudaEventRecord(ev[1], st));
        launch_pass<PASS_E2>(g, Qs, bl, gr, st, sk);
        launch_bnd<PASS_E2>(g, Qs, bd, nbd, st);
        CK(cudaEventRecord(ev[2], st));
        launch_pass<PASS_F3>(g, Qs, bl, gr, st, sk);
        launch_bnd<PASS_F3>(g, Qs, bd, nbd, st);
        CK(cudaEventRecord(ev[3], st));
        launch_pass<PASS_E4>(g, Qs, bl, gr, st, sk);
        launch_bnd<PASS_E4>(g, Qs, bd, nbd, st);
        CK(cudaEventRecord(ev[4], st));
        launch_pass<PASS_F5>(g, Qs, bl, gr, st, sk);
        launch_bnd<PASS_F5>(g, Qs, bd, nbd, st);
        CK(cudaEventRecord(ev[5], st));
        launch_pass<PASS_CRIT>(g, Qs, bl, gr, st, sk);
        launch_bnd<PASS_CRIT>(g, Qs, bd, nbd, st);
        CK(cudaEventRecord(ev[6], st));
        CK(cudaEventSynchronize(ev[6]));
        for (int k = 0; k < 6; k++) {
            float t = 0;
            cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
            acc[k] += t;
        }
        float t = 0;
        cudaEventElapsedTime(&t, ev[0], ev[6]);
        total += t;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    for (int k = 0; k < 6; k++) ms[k] = acc[k] / reps;
    ms[6] = total / reps;
    CK(cudaGetLastError());
    return DMTZ_OK;
}

}  // extern "C"

// =============================================================================
// allocation-free extraction (dmtz_extract_noalloc)
// =============================================================================
namespace {

// byte layout of the fixed scratch: the FieldState arrays of one field, each
// starting on a 256-byte boundary
constexpr i64 kNaV = DMTZ_NOALLOC_MAX_VERTICES;
constexpr i64 na_round(i64 b) { return (b + 255) / 256 * 256; }
constexpr i64 kNaKey = 0;
constexpr i64 kNaLow = kNaKey + na_round(kNaV * 8);
constexpr i64 kNaPv = kNaLow + na_round(kNaV * 2);
constexpr i64 kNaEa2 = kNaPv + na_round(kNaV * 1);
constexpr i64 kNaFp3 = kNaEa2 + na_round(kNaV * 4);
constexpr i64 kNaFa3 = kNaFp3 + na_round(kNaV * 2);
constexpr i64 kNaEup = kNaFa3 + na_round(kNaV * 4);
constexpr i64 kNaFup = kNaEup + na_round(kNaV * 4);
// no criticality array: the export reads the pairing state alone
constexpr i64 kNaBytes = kNaFup + na_round(kNaV * 4);

}  // namespace

// Every array of the gradient state is fully rewritten by the passes before it
// is read, so the contents a previous call left behind need no clearing.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

namespace {
std::mutex g_noalloc_mu;
constexpr int kNaMaxDevices = 64;
void *g_noalloc_addr[kNaMaxDevices] = {};

// device address of the scratch on the current device, looked up once per
// device.  The address belongs to the device's primary context: a
// cudaDeviceReset between calls (which reloads the module) is not supported.
cudaError_t noalloc_scratch(int dev, unsigned char **out) {
    if (dev < 0 || dev >= kNaMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_noalloc_addr[dev] = p;
    }
    *out = (unsigned char *)g_noalloc_addr[dev];
    return cudaSuccess;
}
}  // namespace

extern "C" dmtz_status dmtz_extract_noalloc(int W, int H, int D, const double *data, int32_t *PV, int32_t *PE,
                                            int32_t *PF, int32_t *PT, void *stream) {
    if (W < 2 || H < 2 || D < 2 || !data || !PV || !PE || !PF || !PT) return DMTZ_ERR_ARG;
    const Grid g = make_grid(W, H, D);
    if (g.V > kNaV) return DMTZ_ERR_TOO_LARGE;
    // an error left by the caller's own earlier work stays the caller's: it is
    // reported, not cleared, and nothing is launched
    if (cudaPeekAtLastError() != cudaSuccess) return DMTZ_ERR_CUDA;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return DMTZ_ERR_CUDA;
    unsigned char *base = nullptr;
    if (noalloc_scratch(dev, &base) != cudaSuccess) return DMTZ_ERR_CUDA;
    FieldState s;
    s.val = data;
    s.key = (uint64_t *)(base + kNaKey);
    s.low = (uint16_t *)(base + kNaLow);
    s.pv = (uint8_t *)(base + kNaPv);
    s.ea2 = (uint32_t *)(base + kNaEa2);
    s.fp3 = (uint16_t *)(base + kNaFp3);
    s.fa3 = (uint32_t *)(base + kNaFa3);
    s.eup = (uint32_t *)(base + kNaEup);
    s.fup = (uint32_t *)(base + kNaFup);
    s.crit = nullptr;
    s.tcode = nullptr;
    cudaStream_t st = (cudaStream_t)stream;
    i64 nb;
    const BrickList bl = all_bricks(g, 0, nb);
    const unsigned gb = (unsigned)std::max<i64>(1, std::min<i64>(nb, (i64)persistent_grid() * 2));
    launch_pass<PASS_VERTEX>(g, s, bl, gb, st);
    launch_pass<PASS_E2>(g, s, bl, gb, st);
    launch_pass<PASS_F3>(g, s, bl, gb, st);
    launch_pass<PASS_E4>(g, s, bl, gb, st);
    launch_pass<PASS_F5>(g, s, bl, gb, st);
    k_export<<<grid_for(g.V), kBlock, 0, st>>>(g, s, PV, PE, PF, PT);
    return cudaGetLastError() == cudaSuccess ? DMTZ_OK : DMTZ_ERR_CUDA;
}
