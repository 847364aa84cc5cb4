// pairing_fast.cuh — interior fast path of the pairing passes.
//
// An anchor at 1 <= x,y,z <= dim-2 owns all 26 of its cells and every vertex
// its passes look at (offsets -1..1) exists, so no bounds test is needed.
// Vertex indices are 32-bit here (grids below 2^31 vertices, Grid::small):
// half the integer work of 64-bit ids in the address and tie-break
// arithmetic, which dominates these instruction-bound passes.
// These versions unroll every loop over edge families, triangle slots and
// cofaces at compile time: the topology tables become immediates and each
// "is n below u" test is one shift of a 14-bit mask by a constant.  They
// compute exactly what pass_*_at in pairing.cuh computes (same candidates,
// same argmin rule, same free-target checks); the sweep uses them for interior
// anchors and the generic code for the boundary layer.
#pragma once
#include <utility>

#include "pairing.cuh"

namespace dmtz {
namespace cxt {
#define TOPO_QUAL static constexpr
#include "topology_tables.inc"
#undef TOPO_QUAL

__host__ __device__ constexpr int cdir(int dx, int dy, int dz) {
    return (dx < -1 || dx > 1 || dy < -1 || dy > 1 || dz < -1 || dz > 1) ? -1
                                                                         : TOPO_DIR_LUT[(dx + 1) + 3 * (dy + 1) + 9 * (dz + 1)];
}
__host__ __device__ constexpr int ccx(int c) { return c & 1; }
__host__ __device__ constexpr int ccy(int c) { return (c >> 1) & 1; }
__host__ __device__ constexpr int ccz(int c) { return (c >> 2) & 1; }
// direction from corner c to offset (x, y, z), all relative to the same anchor
__host__ __device__ constexpr int cdir_to(int c, int x, int y, int z) { return cdir(x - ccx(c), y - ccy(c), z - ccz(c)); }
// Candidates in increasing vertex id order.  Every candidate of a selection
// is the anchor plus a compile-time offset (-1..2 per axis), and ids grow with
// (dz, dy, dx) lexicographically, so visiting candidates in that order and
// keeping the first of equal keys (a strict key comparison) takes the
// smallest id among equal values: the (value, id) tie-break of
// compare_vertices (main_3d.cu:1043-1049) without comparing ids.
__host__ __device__ constexpr int lex3(int x, int y, int z) { return (z + 4) * 64 + (y + 4) * 8 + (x + 4); }
__host__ __device__ constexpr int dir_by_id(int r) {
    for (int i = 0; i < 14; i++) {
        int rank = 0;
        for (int j = 0; j < 14; j++)
            rank += lex3(TOPO_DIRS[j][0], TOPO_DIRS[j][1], TOPO_DIRS[j][2]) <
                    lex3(TOPO_DIRS[i][0], TOPO_DIRS[i][1], TOPO_DIRS[i][2]);
        if (rank == r) return i;
    }
    return -1;
}
__host__ __device__ constexpr bool dir_up(int i) { return lex3(TOPO_DIRS[i][0], TOPO_DIRS[i][1], TOPO_DIRS[i][2]) > lex3(0, 0, 0); }
__host__ __device__ constexpr int edge_cand_by_id(int k, int r) {
    for (int i = 0; i < TOPO_EDGE_NCOF[k]; i++) {
        int rank = 0;
        for (int j = 0; j < TOPO_EDGE_NCOF[k]; j++)
            rank += lex3(TOPO_EDGE_THIRD[k][j][0], TOPO_EDGE_THIRD[k][j][1], TOPO_EDGE_THIRD[k][j][2]) <
                    lex3(TOPO_EDGE_THIRD[k][i][0], TOPO_EDGE_THIRD[k][i][1], TOPO_EDGE_THIRD[k][i][2]);
        if (rank == r) return i;
    }
    return -1;
}
__host__ __device__ constexpr int face_cand_by_id(int s, int r) {
    for (int i = 0; i < TOPO_FACE_NCOF[s]; i++) {
        int rank = 0;
        for (int j = 0; j < TOPO_FACE_NCOF[s]; j++)
            rank += lex3(TOPO_FACE_FOURTH[s][j][0], TOPO_FACE_FOURTH[s][j][1], TOPO_FACE_FOURTH[s][j][2]) <
                    lex3(TOPO_FACE_FOURTH[s][i][0], TOPO_FACE_FOURTH[s][i][1], TOPO_FACE_FOURTH[s][i][2]);
        if (rank == r) return i;
    }
    return -1;
}
// index of the corner with offset (x,y,z) among a tet's four corners (-1 if none)
__host__ __device__ constexpr int tet_corner_index(int ts, int x, int y, int z) {
    return (TOPO_TET_V[ts][0] == x + 2 * y + 4 * z)   ? 0
           : (TOPO_TET_V[ts][1] == x + 2 * y + 4 * z) ? 1
           : (TOPO_TET_V[ts][2] == x + 2 * y + 4 * z) ? 2
           : (TOPO_TET_V[ts][3] == x + 2 * y + 4 * z) ? 3
                                                      : -1;
}
}  // namespace cxt

// linear offset of a compile-time displacement
template <int DX, int DY, int DZ>
__device__ __forceinline__ int off(const Grid &g) {
    return DX + DY * g.W + DZ * g.WHi;
}

__device__ __forceinline__ bool key_less32(uint64_t ka, int a, uint64_t kb, int b) {
    return ka < kb || (ka == kb && a < b);
}
// the same order without branches, for the candidate loops of the edge and
// triangle passes: their bodies are short and in most warps some lane takes
// each one, so selecting costs less than branching (measured at 256^3: the
// four passes 8 % faster)
__device__ __forceinline__ bool key_less32_nb(uint64_t ka, int a, uint64_t kb, int b) {
    return (ka < kb) | ((ka == kb) & (a < b));
}

template <int... Is, class F>
__device__ __forceinline__ void static_for(std::integer_sequence<int, Is...>, F &&f) {
    (f(std::integral_constant<int, Is>{}), ...);
}
#define DMTZ_FOR(N, VAR, ...) static_for(std::make_integer_sequence<int, N>{}, [&](auto VAR) __VA_ARGS__)

__device__ __forceinline__ bool bit(uint32_t m, int d) { return (m >> d) & 1u; }

// ---------------------------------------------------------------- pass 1
// s.key holds the order keys of the anchor and its neighbours (the staged
// sweep computes them while staging).  The reference's search starts from
// DBL_MAX with id -1, so a neighbour whose value is DBL_MAX is never taken:
// a strict comparison against that key does the same.
__device__ __forceinline__ void fast_vertex(const Grid &g, const FieldState &s, int v) {
    const uint64_t kv = s.key[v];
    uint64_t bk = DMTZ_KEY_DBL_MAX;
    int bdir = 15;
    uint32_t lm = 0;
    DMTZ_FOR(14, R, {
        constexpr int i = cxt::dir_by_id(decltype(R)::value);
        const uint64_t kn = s.key[v + off<cxt::TOPO_DIRS[i][0], cxt::TOPO_DIRS[i][1], cxt::TOPO_DIRS[i][2]>(g)];
        // below v in (value, id) order; the neighbour's id is above v's iff dir_up
        const bool below = cxt::dir_up(i) ? (kn < kv) : (kn <= kv);
        lm |= below ? (1u << i) : 0u;
        const bool better = below & (kn < bk);
        bk = better ? kn : bk;
        bdir = better ? i : bdir;
    });
    s.low[v] = (uint16_t)lm;
    s.pv[v] = (uint8_t)bdir;
}

// start of the edge and triangle passes' searches: the reference starts from
// DBL_MAX with the largest id, so a candidate whose value is DBL_MAX is taken
// over the start; one above DBL_MAX's key, a strict comparison does the same
#define DMTZ_KEY_ABOVE_DBL_MAX (DMTZ_KEY_DBL_MAX + 1ull)

// ---------------------------------------------------------------- pass 2 / 4 (edges)
// A2 = true: candidates below both endpoints (pass 2); false: between them (pass 4)
template <int K, bool A2>
__device__ __forceinline__ int fast_edge_choice(const Grid &g, const FieldState &s, int v, bool &claimed) {
    constexpr int cp = cxt::TOPO_EDGE_V[K][0], cq = cxt::TOPO_EDGE_V[K][1];
    constexpr int dpq = cxt::TOPO_CORNER_DIR[cp][cq], dqp = cxt::TOPO_CORNER_DIR[cq][cp];
    const int p = v + g.coff32[cp], q = v + g.coff32[cq];
    const uint32_t lp = s.low[p], lq = s.low[q];
    const bool qb = bit(lp, dpq);  // q below p: p is the higher endpoint
    claimed = qb ? (s.pv[p] == dpq) : (s.pv[q] == dqp);
    if (claimed) return -1;
    // candidates: below both endpoints (pass 2), i.e. below the lower one;
    // or below exactly one of them (pass 4), i.e. below the higher and not
    // below the lower one (the order is total)
    uint64_t bk = DMTZ_KEY_ABOVE_DBL_MAX;
    int bj = -1;
    DMTZ_FOR(cxt::TOPO_EDGE_NCOF[K], R, {
        constexpr int j = cxt::edge_cand_by_id(K, decltype(R)::value);
        constexpr int tx = cxt::TOPO_EDGE_THIRD[K][j][0], ty = cxt::TOPO_EDGE_THIRD[K][j][1],
                      tz = cxt::TOPO_EDGE_THIRD[K][j][2];
        constexpr int dp = cxt::cdir_to(cp, tx, ty, tz), dq = cxt::cdir_to(cq, tx, ty, tz);
        const bool ok = A2 ? (bit(lp, dp) & bit(lq, dq)) : (bit(lp, dp) ^ bit(lq, dq));
        const uint64_t kn = s.key[v + off<tx, ty, tz>(g)];
        const bool better = ok & (kn < bk);
        bk = better ? kn : bk;
        bj = better ? j : bj;
    });
    return bj;
}

__device__ __forceinline__ void fast_edge_a2(const Grid &g, const FieldState &s, int v) {
    uint32_t out = 0;
    DMTZ_FOR(7, K, {
        constexpr int k = decltype(K)::value;
        bool claimed;
        const int bj = fast_edge_choice<k, true>(g, s, v, claimed);
        if (bj >= 0) out |= (uint32_t)(bj + 1) << (3 * k);
    });
    s.ea2[v] = out;
}

// is the face (anchor offset, slot) paired after pass 3?
template <int K, int J>
__device__ __forceinline__ bool cof_face_paired3(const Grid &g, const FieldState &s, int v) {
    constexpr int fx = cxt::TOPO_EDGE_COF[K][J][0], fy = cxt::TOPO_EDGE_COF[K][J][1],
                  fz = cxt::TOPO_EDGE_COF[K][J][2], fs = cxt::TOPO_EDGE_COF[K][J][3];
    return bit(s.fp3[v + off<fx, fy, fz>(g)], fs);
}

// pass 4 for one edge slot K of anchor v (an edge pass 2 left unpaired): its
// choice if that triangle is still free, as the slot's bits of eup (0 if none)
template <int K>
__device__ __forceinline__ uint32_t edge_a4_slot(const Grid &g, const FieldState &s, int v) {
    bool claimed;
    const int bj = fast_edge_choice<K, false>(g, s, v, claimed);
    if (bj < 0) return 0u;
    bool taken = false;
    DMTZ_FOR(cxt::TOPO_EDGE_NCOF[K], J, {
        constexpr int j = decltype(J)::value;
        if (bj == j) taken = cof_face_paired3<K, j>(g, s, v);
    });
    return taken ? 0u : (uint32_t)(bj + 1) << (3 * K);
}

// ---------------------------------------------------------------- triangles
// value order of the triangle's corners (j = 0,1,2 by id): lowest / middle
template <int S>
__device__ __forceinline__ void fast_tri_order(const FieldState &s, const uint32_t l[3], int &jlo, int &jmid) {
    constexpr int c0 = cxt::TOPO_FACE_V[S][0], c1 = cxt::TOPO_FACE_V[S][1], c2 = cxt::TOPO_FACE_V[S][2];
    const bool b01 = bit(l[0], cxt::TOPO_CORNER_DIR[c0][c1]);
    const bool b02 = bit(l[0], cxt::TOPO_CORNER_DIR[c0][c2]);
    const bool b12 = bit(l[1], cxt::TOPO_CORNER_DIR[c1][c2]);
    const int r0 = (int)b01 + (int)b02, r1 = (int)(!b01) + (int)b12;
    jlo = r0 == 0 ? 0 : (r1 == 0 ? 1 : 2);
    const int jhi = r0 == 2 ? 0 : (r1 == 2 ? 1 : 2);
    jmid = 3 - jlo - jhi;
}

// does the edge of slot S opposite corner j point (through `arr`) to this triangle?
template <int S>
__device__ __forceinline__ bool edge_points_to_face(const Grid &g, const uint32_t *arr, int v, int j) {
    bool r = false;
    DMTZ_FOR(3, J, {
        constexpr int jj = decltype(J)::value;
        constexpr int ex = cxt::TOPO_FACE_EDGE[S][jj][0], ey = cxt::TOPO_FACE_EDGE[S][jj][1],
                      ez = cxt::TOPO_FACE_EDGE[S][jj][2], ek = cxt::TOPO_FACE_EDGE[S][jj][3],
                      ei = cxt::TOPO_FACE_EDGE[S][jj][4];
        if (j == jj) r = eup_get(arr[v + off<ex, ey, ez>(g)], ek) == ei + 1;
    });
    return r;
}

// argmin over the triangle's cofaces of the fourth vertex, among those with
// "below lo" (A3) or "below mid and above lo" (A5)
template <int S, bool A3>
__device__ __forceinline__ int fast_face_choice(const Grid &g, const FieldState &s, int v, const uint32_t l[3], int jlo,
                                                int jmid) {
    constexpr int c0 = cxt::TOPO_FACE_V[S][0], c1 = cxt::TOPO_FACE_V[S][1], c2 = cxt::TOPO_FACE_V[S][2];
    // candidates: below the lowest corner (pass 3), i.e. below all three; or
    // below the middle and not below the lowest one (pass 5), i.e. below
    // exactly two of the three (the order is total)
    uint64_t bk = DMTZ_KEY_ABOVE_DBL_MAX;
    int bj = -1;
    DMTZ_FOR(cxt::TOPO_FACE_NCOF[S], R, {
        constexpr int j = cxt::face_cand_by_id(S, decltype(R)::value);
        constexpr int nx = cxt::TOPO_FACE_FOURTH[S][j][0], ny = cxt::TOPO_FACE_FOURTH[S][j][1],
                      nz = cxt::TOPO_FACE_FOURTH[S][j][2];
        constexpr int d0 = cxt::cdir_to(c0, nx, ny, nz), d1 = cxt::cdir_to(c1, nx, ny, nz),
                      d2 = cxt::cdir_to(c2, nx, ny, nz);
        const bool b0 = bit(l[0], d0), b1 = bit(l[1], d1), b2 = bit(l[2], d2);
        const bool ok = A3 ? (b0 & b1 & b2) : (((b0 & b1) | (b0 & b2) | (b1 & b2)) & !(b0 & b1 & b2));
        const uint64_t kn = s.key[v + off<nx, ny, nz>(g)];
        const bool better = ok & (kn < bk);
        bk = better ? kn : bk;
        bj = better ? j : bj;
    });
    return bj;
}

template <int S>
__device__ __forceinline__ void load_corner_lows(const Grid &g, const FieldState &s, int v, uint32_t l[3]) {
    constexpr int c0 = cxt::TOPO_FACE_V[S][0], c1 = cxt::TOPO_FACE_V[S][1], c2 = cxt::TOPO_FACE_V[S][2];
    l[0] = s.low[v + off<cxt::ccx(c0), cxt::ccy(c0), cxt::ccz(c0)>(g)];
    l[1] = s.low[v + off<cxt::ccx(c1), cxt::ccy(c1), cxt::ccz(c1)>(g)];
    l[2] = s.low[v + off<cxt::ccx(c2), cxt::ccy(c2), cxt::ccz(c2)>(g)];
}

__device__ __forceinline__ void fast_face_a3(const Grid &g, const FieldState &s, int v) {
    uint32_t out = 0, paired = 0;
    DMTZ_FOR(12, S, {
        constexpr int sl = decltype(S)::value;
        uint32_t l[3];
        load_corner_lows<sl>(g, s, v, l);
        int jlo, jmid;
        fast_tri_order<sl>(s, l, jlo, jmid);
        if (edge_points_to_face<sl>(g, s.ea2, v, jlo)) {
            paired |= 1u << sl;
        } else {
            const int bj = fast_face_choice<sl, true>(g, s, v, l, jlo, jmid);
            if (bj >= 0) {
                out |= (uint32_t)(bj + 1) << (2 * sl);
                paired |= 1u << sl;
            }
        }
    });
    s.fa3[v] = out;
    s.fp3[v] = (uint16_t)paired;
}

// was coface tet J of slot S claimed in pass 3?  Its claimer there is its
// triangle opposite its lowest vertex, which is corner jlo of the triangle.
template <int S, int J>
__device__ __forceinline__ bool cof_tet_claimed3(const Grid &g, const FieldState &s, int v, int jlo) {
    constexpr int tx = cxt::TOPO_FACE_COF[S][J][0], ty = cxt::TOPO_FACE_COF[S][J][1], tz = cxt::TOPO_FACE_COF[S][J][2],
                  ts = cxt::TOPO_FACE_COF[S][J][3];
    bool r = false;
    DMTZ_FOR(3, JL, {
        constexpr int jl = decltype(JL)::value;
        constexpr int c = cxt::TOPO_FACE_V[S][jl];
        constexpr int qi = cxt::tet_corner_index(ts, cxt::ccx(c) - tx, cxt::ccy(c) - ty, cxt::ccz(c) - tz);
        static_assert(qi >= 0, "face corner must be a corner of its coface");
        constexpr int fx = tx + cxt::TOPO_TET_FACE[ts][qi][0], fy = ty + cxt::TOPO_TET_FACE[ts][qi][1],
                      fz = tz + cxt::TOPO_TET_FACE[ts][qi][2], fsl = cxt::TOPO_TET_FACE[ts][qi][3],
                      fci = cxt::TOPO_TET_FACE[ts][qi][4];
        if (jlo == jl) r = fup_get(s.fa3[v + off<fx, fy, fz>(g)], fsl) == fci + 1;
    });
    return r;
}

// pass 5 for one triangle slot S of anchor v (a triangle pass 3 left
// unpaired): unless pass 4 paired it with an edge, its choice if that
// tetrahedron is still free, as the slot's bits of fup (0 if none)
template <int S>
__device__ __forceinline__ uint32_t face_a5_slot(const Grid &g, const FieldState &s, int v) {
    const bool ep = edge_points_to_face<S>(g, s.eup, v, 0) || edge_points_to_face<S>(g, s.eup, v, 1) ||
                    edge_points_to_face<S>(g, s.eup, v, 2);
    if (ep) return 0u;
    uint32_t l[3];
    load_corner_lows<S>(g, s, v, l);
    int jlo, jmid;
    fast_tri_order<S>(s, l, jlo, jmid);
    const int bj = fast_face_choice<S, false>(g, s, v, l, jlo, jmid);
    if (bj < 0) return 0u;
    bool claimed = false;
    DMTZ_FOR(cxt::TOPO_FACE_NCOF[S], J, {
        constexpr int j = decltype(J)::value;
        if (bj == j) claimed = cof_tet_claimed3<S, j>(g, s, v, jlo);
    });
    return claimed ? 0u : (uint32_t)(bj + 1) << (2 * S);
}

// ---------------------------------------------------------------- criticality
__device__ __forceinline__ void fast_crit(const Grid &g, const FieldState &s, int v) {
    uint32_t m = s.pv[v] == 15 ? 1u : 0u;
    const uint32_t eu = s.eup[v], fu = s.fup[v];
    DMTZ_FOR(7, K, {
        constexpr int k = decltype(K)::value;
        constexpr int cp = cxt::TOPO_EDGE_V[k][0], cq = cxt::TOPO_EDGE_V[k][1];
        if (!eup_get(eu, k)) {
            const bool vp = s.pv[v + g.coff32[cp]] == cxt::TOPO_CORNER_DIR[cp][cq] ||
                            s.pv[v + g.coff32[cq]] == cxt::TOPO_CORNER_DIR[cq][cp];
            if (!vp) m |= 1u << (1 + k);
        }
    });
    DMTZ_FOR(12, S, {
        constexpr int sl = decltype(S)::value;
        if (!fup_get(fu, sl)) {
            const bool pe = edge_points_to_face<sl>(g, s.eup, v, 0) || edge_points_to_face<sl>(g, s.eup, v, 1) ||
                            edge_points_to_face<sl>(g, s.eup, v, 2);
            if (!pe) m |= 1u << (8 + sl);
        }
    });
    uint32_t code = 0;
    DMTZ_FOR(6, TS, {
        constexpr int ts = decltype(TS)::value;
        int pj = 7;
        DMTZ_FOR(4, J, {
            constexpr int j = decltype(J)::value;
            constexpr int fx = cxt::TOPO_TET_FACE[ts][j][0], fy = cxt::TOPO_TET_FACE[ts][j][1],
                          fz = cxt::TOPO_TET_FACE[ts][j][2], fsl = cxt::TOPO_TET_FACE[ts][j][3],
                          fci = cxt::TOPO_TET_FACE[ts][j][4];
            if (fup_get(s.fup[v + off<fx, fy, fz>(g)], fsl) == fci + 1) pj = j;
        });
        if (pj == 7) m |= 1u << (20 + ts);
        code |= (uint32_t)pj << (3 * ts);
    });
    s.crit[v] = m;
    if (s.tcode) s.tcode[v] = code;
}

// ---------------------------------------------------------------- brick sweep
enum { PASS_VERTEX = 0, PASS_E2, PASS_F3, PASS_E4, PASS_F5, PASS_CRIT };

// minimum resident blocks per SM the sweep kernels are compiled for: 12
// blocks of 128 threads cap them at 40 registers.  Measured on GB300 at 256^3
// (staged kernels): 16 blocks / 32 registers spill and take 4.98 ms per sweep,
// 12 / 40 take 4.56 ms, 10 / 48 4.68 ms, 8 / 64 4.89 ms.
#ifndef DMTZ_SWEEP_MINB
#define DMTZ_SWEEP_MINB 12
#endif

// the generic (bounds-checked) version of one pass at one anchor
template <int PASS>
__device__ __forceinline__ void pass_at(const Grid &g, const FieldState &s, i64 v, int x, int y, int z) {
    if (PASS == PASS_VERTEX) pass_vertex_at(g, s, v, x, y, z);
    else if (PASS == PASS_E2) pass_edge_a2_at(g, s, v, x, y, z);
    else if (PASS == PASS_F3) pass_face_a3_at(g, s, v, x, y, z);
    else if (PASS == PASS_E4) pass_edge_a4_at(g, s, v, x, y, z);
    else if (PASS == PASS_F5) pass_face_a5_at(g, s, v, x, y, z);
    else {
        uint32_t tc;
        s.crit[v] = crit_mask(g, s, v, x, y, z, &tc);
        if (s.tcode) s.tcode[v] = tc;
    }
}

// ------------------------------------------------------------- staged sweep
// One pass over the anchors of the listed bricks.  With skip_bnd, anchors on
// the grid's surface are left to k_sweep_bnd: in a brick that touches the
// surface, a warp holding both kinds would run the fast and the generic code
// one after the other (the surface is 2 % of the anchors at 256^3 but its
// mixed warps cost a quarter of a sweep).
//
// The interior passes read only anchors at offsets -1..1 (the corner, third-
// and fourth-vertex, edge- and face-anchor tables all stay in that range), so
// a brick's inputs are its anchors plus a one-anchor halo.  k_sweep_sm copies
// the pass's input arrays for that box into shared memory (box rows are
// contiguous in HBM), runs the fast path on box indices -- a Grid whose row
// and plane strides are the box's, so every neighbour offset is a
// compile-time constant -- into box-sized shared output arrays, and writes
// its anchors' outputs back.  Shared-memory latency replaces the L1/L2
// latency of the neighbour loads that stalled the passes.
template <int BX, int BY>
__device__ __forceinline__ Grid box_grid() {
    Grid b;
    b.W = BX;
    b.H = BY;
    b.D = 1;
    b.WH = BX * BY;
    b.small = 1;
    b.WHi = BX * BY;
    DMTZ_FOR(14, I, {
        constexpr int i = decltype(I)::value;
        constexpr int d = cxt::TOPO_DIRS[i][0] + cxt::TOPO_DIRS[i][1] * BX + cxt::TOPO_DIRS[i][2] * BX * BY;
        b.doff32[i] = d;
    });
#pragma unroll
    for (int c8 = 0; c8 < 8; c8++) b.coff32[c8] = (c8 & 1) + ((c8 >> 1) & 1) * BX + ((c8 >> 2) & 1) * BX * BY;
    return b;
}

template <int PASS, int SX, int SY, int SZ>
__global__ void __launch_bounds__(DMTZ_BRICK, DMTZ_SWEEP_MINB) k_sweep_sm(Grid g, FieldState s, BrickList bl,
                                                                        int skip_bnd) {
    static_assert(SX * SY * SZ == DMTZ_BRICK, "a brick is one block");
    constexpr int BX = SX + 2, BY = SY + 2, BZ = SZ + 2, NB = BX * BY * BZ;
    // pass: inputs -> outputs (shared arrays)
    //   0: val -> key low pv        1: low pv key -> ea2 (a)
    //   2: low key ea2 (a) -> fa3 (b) fp3 (c)
    //   3: ea2 (a) low pv key fp3 (c) -> eup (b)
    //   4: eup (a) fa3 (b) fp3 (c) low key -> fup (d)
    //   5: pv eup (a) fup (b) -> crit (d) tcode (e)
    constexpr bool K = PASS <= 4, L = PASS <= 4, PV = PASS != 2 && PASS != 4, A = PASS >= 1, B = PASS >= 2,
                   C = PASS >= 2 && PASS <= 4, DD = PASS >= 4, E = PASS == 5, VAL = PASS == 0;
    __shared__ uint64_t sh_key[K ? NB : 1];

    __shared__ uint16_t sh_low[L ? NB : 1];
    __shared__ uint8_t sh_pv[PV ? NB : 1];
    __shared__ uint32_t sh_a[A ? NB : 1];
    __shared__ uint32_t sh_b[B ? NB : 1];
    __shared__ uint16_t sh_c[C ? NB : 1];
    __shared__ uint32_t sh_d[DD ? NB : 1];
    __shared__ uint32_t sh_e[E ? NB : 1];
    // passes 3 and 4: per slot, the box indices of the anchors whose cell of
    // that slot is still unpaired, and their count
    constexpr bool CMP = PASS == 3 || PASS == 4;
    constexpr int NS = PASS == 3 ? 7 : 12;
    __shared__ uint16_t sh_item[CMP ? NS : 1][CMP ? DMTZ_BRICK : 1];
    __shared__ unsigned sh_cnt[CMP ? NS : 1];
    if (CMP && threadIdx.x < NS) sh_cnt[threadIdx.x] = 0;
    const Grid gb = box_grid<BX, BY>();
    FieldState t;  // box views of the pass's inputs and outputs
    t.val = nullptr;
    t.key = sh_key;
    t.low = sh_low;
    t.pv = sh_pv;
    t.ea2 = sh_a;
    t.fa3 = sh_b;
    t.fp3 = sh_c;
    t.eup = PASS == 3 ? sh_b : sh_a;
    t.fup = PASS == 4 ? sh_d : sh_b;
    t.crit = sh_d;
    t.tcode = (PASS == 5 && s.tcode) ? sh_e : nullptr;
    const int lx = threadIdx.x % SX, ly = (threadIdx.x / SX) % SY, lz = threadIdx.x / (SX * SY);
    const int li = (lx + 1) + BX * ((ly + 1) + BY * (lz + 1));  // this thread's anchor in the box
    const i64 nbr = brick_count(bl);
    // The box entries a thread stages are the same for every brick: their
    // offsets from the box corner (32-bit grids) are computed once.  A brick
    // whose box lies inside the grid (almost all of them) stages without
    // bounds tests, by 32-bit offsets from its corner, and all its anchors
    // take the fast path.
    constexpr int NE = (NB + DMTZ_BRICK - 1) / DMTZ_BRICK;
    int eoff[NE];
#pragma unroll
    for (int k = 0; k < NE; k++) {
        const int e = threadIdx.x + k * DMTZ_BRICK;
        eoff[k] = e % BX + ((e / BX) % BY) * g.W + (e / (BX * BY)) * g.WHi;
    }
    for (i64 b = blockIdx.x; b < nbr; b += gridDim.x) {
        int bx, by, bz;
        brick_coords(bl, b, bx, by, bz);
        const int x0 = bx * SX, y0 = by * SY, z0 = bz * SZ;
        const bool boxin = g.small && x0 >= 1 && y0 >= 1 && z0 >= 1 && x0 + SX < g.W && y0 + SY < g.H && z0 + SZ < g.D;
        const int corner = boxin ? (x0 - 1) + (y0 - 1) * g.W + (z0 - 1) * g.WHi : 0;
        __syncthreads();  // the previous brick's readers are done
        if (boxin) {
#pragma unroll
            for (int k = 0; k < NE; k++) {
                const int e = threadIdx.x + k * DMTZ_BRICK;
                if (k + 1 < NE || e < NB) {
                    const unsigned u = (unsigned)(corner + eoff[k]);
                    if (VAL) sh_key[e] = okey(s.val[u]);
                    if (PASS >= 1 && PASS <= 4) {
                        sh_low[e] = s.low[u];
                        sh_key[e] = s.key[u];
                    }
                    if (PASS == 1 || PASS == 3 || PASS == 5) sh_pv[e] = s.pv[u];
                    if (PASS == 2 || PASS == 3) sh_a[e] = s.ea2[u];
                    if (PASS == 4 || PASS == 5) sh_a[e] = s.eup[u];
                    if (PASS == 3 || PASS == 4) sh_c[e] = s.fp3[u];
                    if (PASS == 4) sh_b[e] = s.fa3[u];
                    if (PASS == 5) sh_b[e] = s.fup[u];
                }
            }
        } else
        for (int e = threadIdx.x; e < NB; e += DMTZ_BRICK) {
            const int ux = x0 - 1 + e % BX, uy = y0 - 1 + (e / BX) % BY, uz = z0 - 1 + e / (BX * BY);
            const bool in = ux >= 0 && uy >= 0 && uz >= 0 && ux < g.W && uy < g.H && uz < g.D;
            const i64 u = in ? ux + (i64)uy * g.W + (i64)uz * g.WH : 0;
            if (VAL) sh_key[e] = in ? okey(s.val[u]) : 0ull;  // pass 0 stages order keys
            if (PASS >= 1 && PASS <= 4) {
                sh_low[e] = in ? s.low[u] : (uint16_t)0;
                sh_key[e] = in ? s.key[u] : 0ull;
            }
            if (PASS == 1 || PASS == 3 || PASS == 5) sh_pv[e] = in ? s.pv[u] : (uint8_t)15;
            if (PASS == 2 || PASS == 3) sh_a[e] = in ? s.ea2[u] : 0u;
            if (PASS == 4 || PASS == 5) sh_a[e] = in ? s.eup[u] : 0u;
            if (PASS == 3 || PASS == 4) sh_c[e] = in ? s.fp3[u] : (uint16_t)0;
            if (PASS == 4) sh_b[e] = in ? s.fa3[u] : 0u;
            if (PASS == 5) sh_b[e] = in ? s.fup[u] : 0u;
        }
        __syncthreads();
        const int x = x0 + lx, y = y0 + ly, z = z0 + lz;
        const bool ingrid = boxin || (x < g.W && y < g.H && z < g.D);
        const bool inner =
            boxin || (ingrid && x >= 1 && y >= 1 && z >= 1 && x <= g.W - 2 && y <= g.H - 2 && z <= g.D - 2);
        const i64 v = boxin ? (i64)(unsigned)(corner + (lx + 1) + (ly + 1) * g.W + (lz + 1) * g.WHi)
                            : x + (i64)y * g.W + (i64)z * g.WH;
        if constexpr (CMP) {
            // The second edge and triangle passes act on the cells the first
            // ones left unpaired (about one in ten), so a warp running slot by
            // slot over its anchors would run every slot's body with a few
            // lanes each.  Instead each slot's pending anchors are listed and
            // its body runs on consecutive threads; a slot's result bits go
            // into the anchor's output word by a shared-memory OR.  Slot s's
            // list starts at warp s mod 4, so the bodies spread over the warps.
            uint32_t need = 0;
            if (inner) {
                if (PASS == 3) {
                    const uint32_t a2 = sh_a[li];
                    sh_b[li] = a2;
                    DMTZ_FOR(7, K, {
                        constexpr int k = decltype(K)::value;
                        need |= eup_get(a2, k) ? 0u : 1u << k;
                    });
                } else {
                    sh_d[li] = sh_b[li];
                    need = ~(uint32_t)sh_c[li] & 0xFFFu;
                }
            }
            const unsigned lane = threadIdx.x & 31u;
            DMTZ_FOR(NS, S, {
                constexpr int sl = decltype(S)::value;
                const bool nd = bit(need, sl);
                const unsigned m = __ballot_sync(0xffffffffu, nd);
                if (m) {
                    unsigned base = 0;
                    if (lane == 0) base = atomicAdd(&sh_cnt[sl], (unsigned)__popc(m));
                    base = __shfl_sync(0xffffffffu, base, 0);
                    if (nd) sh_item[sl][base + (unsigned)__popc(m & ((1u << lane) - 1u))] = (uint16_t)li;
                }
            });
            __syncthreads();
            DMTZ_FOR(NS, S, {
                constexpr int sl = decltype(S)::value;
                const unsigned r = (threadIdx.x + DMTZ_BRICK - 32 * (sl % 4)) % DMTZ_BRICK;
                const bool mine = r < sh_cnt[sl];
                // a vote is warp-uniform: warps without items branch around
                // the body instead of running it under a false predicate
                if (__any_sync(0xffffffffu, mine) && mine) {
                    const int a = sh_item[sl][r];
                    if constexpr (PASS == 3) {
                        const uint32_t bits = edge_a4_slot<sl>(gb, t, a);
                        if (bits) atomicOr(&sh_b[a], bits);
                    } else {
                        const uint32_t bits = face_a5_slot<sl>(gb, t, a);
                        if (bits) atomicOr(&sh_d[a], bits);
                    }
                }
            });
            __syncthreads();
            if (threadIdx.x < NS) sh_cnt[threadIdx.x] = 0;  // read by no thread before the next brick's barriers
            if (inner) {
                if (PASS == 3) s.eup[v] = sh_b[li];
                else s.fup[v] = sh_d[li];
            } else if (ingrid && !skip_bnd) {
                pass_at<PASS>(g, s, v, x, y, z);
            }
        } else if (inner) {
            if (PASS == 0) {
                fast_vertex(gb, t, li);
                s.key[v] = sh_key[li];
                s.low[v] = sh_low[li];
                s.pv[v] = sh_pv[li];
            } else if (PASS == 1) {
                fast_edge_a2(gb, t, li);
                s.ea2[v] = sh_a[li];
            } else if (PASS == 2) {
                fast_face_a3(gb, t, li);
                s.fa3[v] = sh_b[li];
                s.fp3[v] = sh_c[li];
            } else {
                fast_crit(gb, t, li);
                s.crit[v] = sh_d[li];
                if (s.tcode) s.tcode[v] = sh_e[li];
            }
        } else if (ingrid && !skip_bnd) {
            pass_at<PASS>(g, s, v, x, y, z);
        }
    }
}

// one pass over a list of surface anchors (dense warps, generic code)
template <int PASS>
__global__ void __launch_bounds__(256) k_sweep_bnd(Grid g, FieldState s, const i64 *list, i64 n) {
    for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (i64)gridDim.x * blockDim.x) {
        const i64 v = list[i];
        int x, y, z;
        decode_v(g, v, x, y, z);
        pass_at<PASS>(g, s, v, x, y, z);
    }
}

// the anchors on the grid's surface (any coordinate 0 or dim-1), one warp
// atomic per warp
__global__ void k_bnd_list(Grid g, i64 *list, unsigned long long *n) {
    const i64 v = (i64)blockIdx.x * blockDim.x + threadIdx.x;
    bool on = false;
    if (v < g.V) {
        int x, y, z;
        decode_v(g, v, x, y, z);
        on = x == 0 || y == 0 || z == 0 || x == g.W - 1 || y == g.H - 1 || z == g.D - 1;
    }
    const unsigned mask = __ballot_sync(0xffffffffu, on);
    if (!mask) return;
    const unsigned lane = threadIdx.x & 31;
    unsigned long long base = 0;
    if (lane == (unsigned)(__ffs(mask) - 1)) base = atomicAdd(n, (unsigned long long)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, __ffs(mask) - 1);
    if (on) list[base + __popc(mask & ((1u << lane) - 1u))] = v;
}

}  // namespace dmtz

namespace dmtz {
template <int PASS>
inline void launch_bnd(const Grid &g, const FieldState &s, const i64 *list, i64 n, cudaStream_t st) {
    if (n <= 0) return;
    const unsigned gr = (unsigned)std::min<i64>((n + 255) / 256, 65535);
    k_sweep_bnd<PASS><<<gr, 256, 0, st>>>(g, s, list, n);
}
// launch one pass over a brick list with the list's brick shape
template <int PASS>
inline void launch_pass(const Grid &g, const FieldState &s, const BrickList &bl, unsigned grid, cudaStream_t st,
                        int skip_bnd = 0) {
    switch (bl.shape) {
    case 1: k_sweep_sm<PASS, 16, 4, 2><<<grid, DMTZ_BRICK, 0, st>>>(g, s, bl, skip_bnd); break;
    case 2: k_sweep_sm<PASS, 32, 2, 2><<<grid, DMTZ_BRICK, 0, st>>>(g, s, bl, skip_bnd); break;
    default: k_sweep_sm<PASS, 8, 4, 4><<<grid, DMTZ_BRICK, 0, st>>>(g, s, bl, skip_bnd); break;
    }
}
}  // namespace dmtz
