// pairing.cuh — the discrete gradient (five greedy pairing passes) on sm_103a.
//
// Reference: processVertices (main_3d.cu:1930-1988), edgePairingKernel
// (:1990-2113) and trianglePairingKernel (:2197-2316), run in the order
// vertices, edges(a2=0), triangles(a2=0), edges(a2=1), triangles(a2=1).
//
// Each reference pass loops 14x14 (edges) or 14x14x14 (triangles) times to
// find the common neighbours of a cell's vertices; here the candidates come
// from the coface tables and the "below" tests from one 14-bit mask per
// vertex, so every pass is a short table walk.  The passes keep the
// reference's selection rule exactly: argmin of (value, id) over the
// candidates, starting from (DBL_MAX, INT_MAX) (or id -1 for the vertex
// pass), and a candidate is taken only when the target cell is still free.
// Within one pass no two cells can claim the same target (a triangle is
// claimed by its top two vertices' edge in pass 2 and by its (max,min) edge
// in pass 4; a tetrahedron by its top three vertices' triangle in pass 3 and
// by the triangle without its third-highest vertex in pass 5), so the passes
// are race-free and deterministic.
#pragma once
#include "dmtz_common.cuh"

namespace dmtz {

__device__ __forceinline__ bool key_less(uint64_t ka, i64 a, uint64_t kb, i64 b) {
    return ka < kb || (ka == kb && a < b);
}

// Pass 1: order keys, lower-neighbour masks, steepest descent.
__device__ __forceinline__ void pass_vertex_at(const Grid &g, const FieldState &s, i64 v, int x, int y, int z) {
    const uint64_t kv = okey(s.val[v]);
    uint64_t bk = DMTZ_KEY_DBL_MAX;
    i64 bid = -1;
    int bdir = 15;
    uint32_t lm = 0;
#pragma unroll
    for (int i = 0; i < 14; i++) {
        if (!inb(g, x + TOPO_DIRS[i][0], y + TOPO_DIRS[i][1], z + TOPO_DIRS[i][2])) continue;
        const i64 nb = v + g.doff[i];
        const uint64_t kn = okey(s.val[nb]);
        if (key_less(kn, nb, kv, v)) {
            lm |= 1u << i;
            if (key_less(kn, nb, bk, bid)) {
                bk = kn;
                bid = nb;
                bdir = i;
            }
        }
    }
    s.key[v] = kv;
    s.low[v] = (uint16_t)lm;
    s.pv[v] = (uint8_t)bdir;
}

// corner c of anchor v: linear index and coordinates
struct Corner {
    i64 id;
    int x, y, z;
};
__device__ __forceinline__ Corner corner_at(const Grid &g, i64 v, int x, int y, int z, int c) {
    Corner r;
    int dx, dy, dz;
    corner_xyz(c, dx, dy, dz);
    r.id = v + g.coff[c];
    r.x = x + dx; r.y = y + dy; r.z = z + dz;
    return r;
}
// is vertex b below adjacent vertex a (direction from a to b = d)?
__device__ __forceinline__ bool below_dir(const uint16_t *low, i64 a, int d) { return (low[a] >> d) & 1; }

// Pass 2: edge -> triangle, candidates below both endpoints (a2 = 0).
__device__ __forceinline__ void pass_edge_a2_at(const Grid &g, const FieldState &s, i64 v, int x, int y, int z) {
    uint32_t out = 0;
    for (int k = 0; k < 7; k++) {
        int mx, my, mz;
        edge_extent(k, mx, my, mz);
        if (!cell_ok(g, x, y, z, mx, my, mz)) continue;
        const int cp = TOPO_EDGE_V[k][0], cq = TOPO_EDGE_V[k][1];
        const Corner p = corner_at(g, v, x, y, z, cp), q = corner_at(g, v, x, y, z, cq);
        const int dpq = TOPO_CORNER_DIR[cp][cq], dqp = TOPO_CORNER_DIR[cq][cp];
        const bool q_below = below_dir(s.low, p.id, dpq);
        const Corner hi = q_below ? p : q, lo = q_below ? q : p;
        const int dhl = q_below ? dpq : dqp;
        if (s.pv[hi.id] == dhl) continue;  // paired with its higher vertex in pass 1
        uint64_t bk = DMTZ_KEY_DBL_MAX;
        i64 bid = INT_MAX;
        int bj = -1;
        const int nc = TOPO_EDGE_NCOF[k];
        for (int j = 0; j < nc; j++) {
            const int nx = x + TOPO_EDGE_THIRD[k][j][0], ny = y + TOPO_EDGE_THIRD[k][j][1],
                      nz = z + TOPO_EDGE_THIRD[k][j][2];
            if (!inb(g, nx, ny, nz)) continue;
            const int d = dir_of(nx - lo.x, ny - lo.y, nz - lo.z);
            if (!below_dir(s.low, lo.id, d)) continue;  // must be below both endpoints
            const i64 nb = nx + (i64)ny * g.W + (i64)nz * g.WH;
            const uint64_t kn = s.key[nb];
            if (key_less(kn, nb, bk, bid)) {
                bk = kn;
                bid = nb;
                bj = j;
            }
        }
        if (bj >= 0) out |= (uint32_t)(bj + 1) << (3 * k);
    }
    s.ea2[v] = out;
}

// value order of a triangle's three corners (given in id order j = 0,1,2):
// returns the corner index j of the lowest / middle / highest vertex
__device__ __forceinline__ void tri_order(const uint16_t *low, const Corner c[3], int &jlo, int &jmid, int &jhi) {
    const bool b01 = below_dir(low, c[0].id, dir_of(c[1].x - c[0].x, c[1].y - c[0].y, c[1].z - c[0].z));
    const bool b02 = below_dir(low, c[0].id, dir_of(c[2].x - c[0].x, c[2].y - c[0].y, c[2].z - c[0].z));
    const bool b12 = below_dir(low, c[1].id, dir_of(c[2].x - c[1].x, c[2].y - c[1].y, c[2].z - c[1].z));
    // rank = number of vertices below
    const int r0 = (int)b01 + (int)b02;
    const int r1 = (int)(!b01) + (int)b12;
    const int r2 = (int)(!b02) + (int)(!b12);
    jlo = r0 == 0 ? 0 : (r1 == 0 ? 1 : 2);
    jhi = r0 == 2 ? 0 : (r1 == 2 ? 1 : 2);
    jmid = 3 - jlo - jhi;
    (void)r2;
}

// Pass 3: triangle -> tetrahedron, candidates below all three (a2 = 0).
__device__ __forceinline__ void pass_face_a3_at(const Grid &g, const FieldState &s, i64 v, int x, int y, int z) {
    uint32_t out = 0;
    uint32_t paired = 0;
    for (int sl = 0; sl < 12; sl++) {
        int mx, my, mz;
        face_extent(sl, mx, my, mz);
        if (!cell_ok(g, x, y, z, mx, my, mz)) continue;
        Corner c[3];
        for (int j = 0; j < 3; j++) c[j] = corner_at(g, v, x, y, z, TOPO_FACE_V[sl][j]);
        int jlo, jmid, jhi;
        tri_order(s.low, c, jlo, jmid, jhi);
        // claimed in pass 2 by the edge of its two highest vertices?
        const signed char *fe = TOPO_FACE_EDGE[sl][jlo];
        const i64 ea = v + fe[0] + (i64)fe[1] * g.W + (i64)fe[2] * g.WH;
        if (eup_get(s.ea2[ea], fe[3]) == fe[4] + 1) {
            paired |= 1u << sl;
            continue;
        }
        const Corner lo = c[jlo];
        uint64_t bk = DMTZ_KEY_DBL_MAX;
        i64 bid = INT_MAX;
        int bj = -1;
        const int nc = TOPO_FACE_NCOF[sl];
        for (int j = 0; j < nc; j++) {
            const int nx = x + TOPO_FACE_FOURTH[sl][j][0], ny = y + TOPO_FACE_FOURTH[sl][j][1],
                      nz = z + TOPO_FACE_FOURTH[sl][j][2];
            if (!inb(g, nx, ny, nz)) continue;
            const int d = dir_of(nx - lo.x, ny - lo.y, nz - lo.z);
            if (!below_dir(s.low, lo.id, d)) continue;
            const i64 nb = nx + (i64)ny * g.W + (i64)nz * g.WH;
            const uint64_t kn = s.key[nb];
            if (key_less(kn, nb, bk, bid)) {
                bk = kn;
                bid = nb;
                bj = j;
            }
        }
        if (bj >= 0) {
            out |= (uint32_t)(bj + 1) << (2 * sl);
            paired |= 1u << sl;
        }
    }
    s.fa3[v] = out;
    s.fp3[v] = (uint16_t)paired;
}

// Pass 4: still-unpaired edges -> triangle whose third vertex lies between
// the endpoints (a2 = 1), if that triangle is still free.
__device__ __forceinline__ void pass_edge_a4_at(const Grid &g, const FieldState &s, i64 v, int x, int y, int z) {
    const uint32_t a2 = s.ea2[v];
    uint32_t out = a2;
    for (int k = 0; k < 7; k++) {
        int mx, my, mz;
        edge_extent(k, mx, my, mz);
        if (!cell_ok(g, x, y, z, mx, my, mz)) continue;
        if (eup_get(a2, k)) continue;
        const int cp = TOPO_EDGE_V[k][0], cq = TOPO_EDGE_V[k][1];
        const Corner p = corner_at(g, v, x, y, z, cp), q = corner_at(g, v, x, y, z, cq);
        const int dpq = TOPO_CORNER_DIR[cp][cq], dqp = TOPO_CORNER_DIR[cq][cp];
        const bool q_below = below_dir(s.low, p.id, dpq);
        const Corner hi = q_below ? p : q, lo = q_below ? q : p;
        const int dhl = q_below ? dpq : dqp;
        if (s.pv[hi.id] == dhl) continue;
        uint64_t bk = DMTZ_KEY_DBL_MAX;
        i64 bid = INT_MAX;
        int bj = -1;
        const int nc = TOPO_EDGE_NCOF[k];
        for (int j = 0; j < nc; j++) {
            const int nx = x + TOPO_EDGE_THIRD[k][j][0], ny = y + TOPO_EDGE_THIRD[k][j][1],
                      nz = z + TOPO_EDGE_THIRD[k][j][2];
            if (!inb(g, nx, ny, nz)) continue;
            const bool below_hi = below_dir(s.low, hi.id, dir_of(nx - hi.x, ny - hi.y, nz - hi.z));
            const bool below_lo = below_dir(s.low, lo.id, dir_of(nx - lo.x, ny - lo.y, nz - lo.z));
            if (!(below_hi && !below_lo)) continue;  // exactly one endpoint above it
            const i64 nb = nx + (i64)ny * g.W + (i64)nz * g.WH;
            const uint64_t kn = s.key[nb];
            if (key_less(kn, nb, bk, bid)) {
                bk = kn;
                bid = nb;
                bj = j;
            }
        }
        if (bj < 0) continue;
        const signed char *cf = TOPO_EDGE_COF[k][bj];
        const i64 fa = v + cf[0] + (i64)cf[1] * g.W + (i64)cf[2] * g.WH;
        if ((s.fp3[fa] >> cf[3]) & 1) continue;  // triangle already paired
        out |= (uint32_t)(bj + 1) << (3 * k);
    }
    s.eup[v] = out;
}

// Pass 5: still-unpaired triangles -> tetrahedron whose fourth vertex is
// below exactly two of the three (a2 = 1), if that tetrahedron is still free.
__device__ __forceinline__ void pass_face_a5_at(const Grid &g, const FieldState &s, i64 v, int x, int y, int z) {
    const uint32_t a3 = s.fa3[v];
    const uint32_t p3 = s.fp3[v];
    uint32_t out = a3;
    for (int sl = 0; sl < 12; sl++) {
        int mx, my, mz;
        face_extent(sl, mx, my, mz);
        if (!cell_ok(g, x, y, z, mx, my, mz)) continue;
        if ((p3 >> sl) & 1) continue;
        // paired with an edge in pass 4?
        bool edge_paired = false;
        for (int j = 0; j < 3; j++) {
            const signed char *fe = TOPO_FACE_EDGE[sl][j];
            const i64 ea = v + fe[0] + (i64)fe[1] * g.W + (i64)fe[2] * g.WH;
            if (eup_get(s.eup[ea], fe[3]) == fe[4] + 1) edge_paired = true;
        }
        if (edge_paired) continue;
        Corner c[3];
        for (int j = 0; j < 3; j++) c[j] = corner_at(g, v, x, y, z, TOPO_FACE_V[sl][j]);
        int jlo, jmid, jhi;
        tri_order(s.low, c, jlo, jmid, jhi);
        const Corner lo = c[jlo], mid = c[jmid];
        uint64_t bk = DMTZ_KEY_DBL_MAX;
        i64 bid = INT_MAX;
        int bj = -1;
        const int nc = TOPO_FACE_NCOF[sl];
        for (int j = 0; j < nc; j++) {
            const int nx = x + TOPO_FACE_FOURTH[sl][j][0], ny = y + TOPO_FACE_FOURTH[sl][j][1],
                      nz = z + TOPO_FACE_FOURTH[sl][j][2];
            if (!inb(g, nx, ny, nz)) continue;
            const bool below_mid = below_dir(s.low, mid.id, dir_of(nx - mid.x, ny - mid.y, nz - mid.z));
            const bool below_lo = below_dir(s.low, lo.id, dir_of(nx - lo.x, ny - lo.y, nz - lo.z));
            if (!(below_mid && !below_lo)) continue;  // below exactly two of the three
            const i64 nb = nx + (i64)ny * g.W + (i64)nz * g.WH;
            const uint64_t kn = s.key[nb];
            if (key_less(kn, nb, bk, bid)) {
                bk = kn;
                bid = nb;
                bj = j;
            }
        }
        if (bj < 0) continue;
        // is the tetrahedron already paired by pass 3?  Its only possible
        // claimer there is the triangle of its top three vertices, i.e. the
        // one opposite its lowest vertex, which is `lo`.
        const signed char *tc = TOPO_FACE_COF[sl][bj];
        const int tx = x + tc[0], ty = y + tc[1], tz = z + tc[2], ts = tc[3];
        const int ldx = lo.x - tx, ldy = lo.y - ty, ldz = lo.z - tz;
        const int lc = ldx + 2 * ldy + 4 * ldz;
        int jj = 0;
        for (int q = 0; q < 4; q++)
            if (TOPO_TET_V[ts][q] == lc) jj = q;
        const signed char *tf = TOPO_TET_FACE[ts][jj];
        const i64 fa = (tx + tf[0]) + (i64)(ty + tf[1]) * g.W + (i64)(tz + tf[2]) * g.WH;
        if (fup_get(s.fa3[fa], tf[3]) == tf[4] + 1) continue;
        out |= (uint32_t)(bj + 1) << (2 * sl);
    }
    s.fup[v] = out;
}

// Critical cells of one anchor (unpaired cells), bit layout of FieldState::crit;
// *tc receives the tetrahedra's pairing codes (FieldState::tcode).
__device__ __forceinline__ uint32_t crit_mask(const Grid &g, const FieldState &s, i64 v, int x, int y, int z,
                                              uint32_t *tc) {
    uint32_t m = 0;
    if (s.pv[v] == 15) m |= 1u;
    const uint32_t eu = s.eup[v];
    for (int k = 0; k < 7; k++) {
        int mx, my, mz;
        edge_extent(k, mx, my, mz);
        if (!cell_ok(g, x, y, z, mx, my, mz)) continue;
        if (eup_get(eu, k)) continue;
        const int cp = TOPO_EDGE_V[k][0], cq = TOPO_EDGE_V[k][1];
        const i64 p = v + g.coff[cp], q = v + g.coff[cq];
        if (s.pv[p] == TOPO_CORNER_DIR[cp][cq] || s.pv[q] == TOPO_CORNER_DIR[cq][cp]) continue;
        m |= 1u << (1 + k);
    }
    const uint32_t fu = s.fup[v];
    for (int sl = 0; sl < 12; sl++) {
        int mx, my, mz;
        face_extent(sl, mx, my, mz);
        if (!cell_ok(g, x, y, z, mx, my, mz)) continue;
        if (fup_get(fu, sl)) continue;
        bool pe = false;
        for (int j = 0; j < 3; j++) {
            const signed char *fe = TOPO_FACE_EDGE[sl][j];
            const i64 ea = v + fe[0] + (i64)fe[1] * g.W + (i64)fe[2] * g.WH;
            if (eup_get(s.eup[ea], fe[3]) == fe[4] + 1) pe = true;
        }
        if (!pe) m |= 1u << (8 + sl);
    }
    uint32_t code = 0x3FFFFu;  // all seven
    if (cell_ok(g, x, y, z, 1, 1, 1)) {
        for (int ts = 0; ts < 6; ts++) {
            int pj = 7;
            for (int j = 0; j < 4; j++) {
                const signed char *tf = TOPO_TET_FACE[ts][j];
                const i64 fa = v + tf[0] + (i64)tf[1] * g.W + (i64)tf[2] * g.WH;
                if (fup_get(s.fup[fa], tf[3]) == tf[4] + 1) pj = j;
            }
            if (pj == 7) m |= 1u << (20 + ts);
            code = (code & ~(7u << (3 * ts))) | ((uint32_t)pj << (3 * ts));
        }
    }
    *tc = code;
    return m;
}

}  // namespace dmtz

namespace dmtz {

// ---------------------------------------------------------------------------
// Brick-driven sweeps.  Anchors are grouped in bricks of 128 (x fastest, one
// 128-thread block per brick; shape chosen by the autotuner, 8 x 4 x 4 by
// default).  A sweep runs over an explicit list of
// bricks (packed bx | by << 11 | bz << 22) or, with list == nullptr, over all
// bricks of the grid.  Blocks stride over the list, so the grid size does not
// depend on its length and the length can stay on the device.
// ---------------------------------------------------------------------------
#define DMTZ_BX 8
#define DMTZ_BY 4
#define DMTZ_BZ 4
#define DMTZ_BRICK (DMTZ_BX * DMTZ_BY * DMTZ_BZ)

struct BrickList {
    const uint32_t *list;           // packed brick coordinates, or nullptr for all bricks
    const unsigned long long *n;    // number of listed bricks (device), when list != nullptr
    int nbx, nby, nbz;              // bricks per axis
    int shape;                      // brick shape index (DMTZ_SHAPES)
    FDiv dbx, dby;                  // division by nbx and nby (brick index -> coordinates)
};
// brick shapes (anchors per brick along x, y, z); each is one 128-thread block
#define DMTZ_NSHAPES 3
static const int DMTZ_SHAPES[DMTZ_NSHAPES][3] = {{8, 4, 4}, {16, 4, 2}, {32, 2, 2}};

__device__ __forceinline__ i64 brick_count(const BrickList &bl) {
    return bl.list ? (i64)*bl.n : (i64)bl.nbx * bl.nby * bl.nbz;
}
__device__ __forceinline__ void brick_coords(const BrickList &bl, i64 b, int &bx, int &by, int &bz) {
    if (bl.list) {
        const uint32_t e = bl.list[b];
        bx = e & 0x7FF;
        by = (e >> 11) & 0x7FF;
        bz = e >> 22;
    } else {  // every thread of the block decodes the same index: multiply-high, not division
        const unsigned long long u = (unsigned long long)b, q = fdiv(bl.dbx, u), r = fdiv(bl.dby, q);
        bx = (int)(u - q * (unsigned long long)bl.nbx);
        by = (int)(q - r * (unsigned long long)bl.nby);
        bz = (int)r;
    }
}

}  // namespace dmtz
