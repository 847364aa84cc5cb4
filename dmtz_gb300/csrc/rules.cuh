// rules.cuh — the reference's fix rules, separatrix checks and value update.
//
// The fix rules (fix_minimum :2554-2586, fix_saddle :2588-3037, fix_2saddle
// :3039-3983, fix_maximum :3985-4303, fix_as_vpath :5135-5244, fix_ds_vpath
// :5246-5295) are a case analysis over the reference's union-valued pairing
// arrays.  They are restated here branch for branch, including the
// reference's quirks (shadowed variables, if/if chains, ids of one dimension
// read as another), on top of accessors that rebuild paired_vertices /
// _edges / _faces / _tetrahedras values from the packed gradient.
//
// A rule "lowers" a vertex: it asks for d_deltaBuffer[v] = get_delta(v).
// get_delta depends only on v's own value and counter, which no rule
// modifies, so the reference's atomic-max / store into the delta buffer is
// the same as set membership: a request bit per vertex (atomicOr) plus a list
// of newly requested vertices.  The value is computed once, when applied.
//
// Any index the reference would read or write outside its allocation is not
// performed; it sets bit 0 of the error word instead.
#pragma once
#include "dmtz_common.cuh"

namespace dmtz {

enum { ERR_OOB = 1, ERR_WALK = 2 };

// The fix rules are long, branchy code run by few lanes of a warp at a time;
// with their id and pairing accessors inlined at every call site the fix
// kernel outgrew the instruction cache (ncu: warps stalled on instruction
// fetch).  The accessors are therefore compiled once and called.
#define DMTZ_SHARED_CODE __noinline__

struct RuleCtx {
    Grid g;
    FieldState P;      // original field gradient
    FieldState Q;      // decompressed field gradient
    const double *f;   // original values
    const double *gv;  // decompressed values (read-only during the rules)
    const int *cnt;    // delta_counter
    double bound;
    int edit_type;
    uint32_t *reqbits;  // request bit per vertex
    i64 *reqlist;       // newly requested vertices
    unsigned long long *reqn;
    i64 reqcap;
    int *err;
    unsigned long long *progress;  // set when an update changes a value or an edit counter
    double range;                  // max - min of the original field
};

// --------------------------------------------------------------- literal id arithmetic
// getVertexIDsFromEdgeID (main_3d.cu:1760-1900) for any id; (a > b)
__device__ DMTZ_SHARED_CODE void edge_verts(const Grid &g, i64 e, i64 &a, i64 &b) {
    const i64 W = g.W, H = g.H, D = g.D;
    int k = -1;
    for (int i = 0; i < 7; i++)
        if (e < g.eoff[i + 1]) {
            k = i;
            break;
        }
    if (k < 0) {
        a = b = -1;
        return;
    }
    const i64 r = e - g.eoff[k];
    i64 x = 0, y = 0, z = 0, x1 = 0, y1 = 0, z1 = 0;
    switch (k) {
    case 0: z = r / ((W - 1) * H); y = (r % ((W - 1) * H)) / (W - 1); x = r % (W - 1);
            x1 = x + 1; y1 = y; z1 = z; break;
    case 1: z = r / (W * (H - 1)); x = (r % (W * (H - 1))) / (H - 1); y = r % (H - 1);
            x1 = x; y1 = y + 1; z1 = z; break;
    case 2: y = r / (W * (D - 1)); x = (r % (W * (D - 1))) / (D - 1); z = r % (D - 1);
            x1 = x; y1 = y; z1 = z + 1; break;
    case 3: { i64 z2 = r / ((W - 1) * (H - 1)), y2 = (r % ((W - 1) * (H - 1))) / (W - 1), x2 = r % (W - 1);
              x = x2 + 1; y = y2; z = z2; x1 = x2; y1 = y2 + 1; z1 = z2; } break;
    case 4: { i64 x2 = r / ((H - 1) * (D - 1)), y2 = (r % ((H - 1) * (D - 1))) / (D - 1), z2 = r % (D - 1);
              x = x2; y = y2; z = z2; x1 = x2; y1 = y2 + 1; z1 = z2 + 1; } break;
    case 5: { i64 y2 = r / ((W - 1) * (D - 1)), z2 = (r % ((W - 1) * (D - 1))) / (W - 1), x2 = r % (W - 1);
              x = x2 + 1; y = y2; z = z2; x1 = x2; y1 = y2; z1 = z2 + 1; } break;
    default: { i64 z2 = r / ((W - 1) * (H - 1)), y2 = (r % ((W - 1) * (H - 1))) / (W - 1), x2 = r % (W - 1);
               x = x2 + 1; y = y2; z = z2; x1 = x2; y1 = y2 + 1; z1 = z2 + 1; } break;
    }
    i64 i1 = x + y * W + z * W * H, i2 = x1 + y1 * W + z1 * W * H;
    a = i1 > i2 ? i1 : i2;
    b = i1 > i2 ? i2 : i1;
}

__device__ __forceinline__ void sort_desc3(i64 &a, i64 &b, i64 &c) {
    i64 t;
    if (a < b) { t = a; a = b; b = t; }
    if (a < c) { t = a; a = c; c = t; }
    if (b < c) { t = b; b = c; c = t; }
}

// getVerticesFromTriangleID (main_3d.cu:425-565) for any id, sorted descending
__device__ DMTZ_SHARED_CODE void tri_verts(const Grid &g, i64 t, i64 &a, i64 &b, i64 &c) {
    const i64 W = g.W, H = g.H, D = g.D, WH = W * H;
    i64 v1 = 0, v2 = 0, v3 = 0, base, mx, my, mz;
    if (t < 2 * D * (W - 1) * (H - 1)) {
        base = t / 2; mz = base / ((W - 1) * (H - 1)); my = (base % ((W - 1) * (H - 1))) / (W - 1); mx = base % (W - 1);
        if (t % 2 == 0) { v1 = mx + my * W + mz * WH; v2 = mx + 1 + my * W + mz * WH; v3 = mx + (my + 1) * W + mz * WH; }
        else { v1 = mx + 1 + (my + 1) * W + mz * WH; v2 = mx + 1 + my * W + mz * WH; v3 = mx + (my + 1) * W + mz * WH; }
    } else if ((t -= 2 * D * (W - 1) * (H - 1)) < 2 * W * (H - 1) * (D - 1)) {
        base = t / 2; mx = base / ((H - 1) * (D - 1)); my = (base % ((H - 1) * (D - 1))) / (D - 1); mz = base % (D - 1);
        if (t % 2 == 0) { v1 = mx + my * W + mz * WH; v2 = mx + (my + 1) * W + mz * WH; v3 = mx + (my + 1) * W + (mz + 1) * WH; }
        else { v1 = mx + my * W + mz * WH; v2 = mx + my * W + (mz + 1) * WH; v3 = mx + (my + 1) * W + (mz + 1) * WH; }
    } else if ((t -= 2 * W * (H - 1) * (D - 1)) < 2 * H * (W - 1) * (D - 1)) {
        base = t / 2; my = base / ((W - 1) * (D - 1)); mz = (base % ((W - 1) * (D - 1))) / (W - 1); mx = base % (W - 1);
        if (t % 2 == 0) { v1 = mx + my * W + mz * WH; v2 = mx + 1 + my * W + mz * WH; v3 = mx + my * W + (mz + 1) * WH; }
        else { v1 = mx + 1 + my * W + mz * WH; v2 = mx + my * W + (mz + 1) * WH; v3 = mx + 1 + my * W + (mz + 1) * WH; }
    } else {
        t -= 2 * H * (W - 1) * (D - 1);
        base = t / 6; mz = base / ((W - 1) * (H - 1)); my = (base % ((W - 1) * (H - 1))) / (W - 1); mx = base % (W - 1);
        const i64 o = mx + my * W + mz * WH;
        switch (t % 6) {
        case 0: v1 = o; v2 = o + 1; v3 = o + W + WH; break;
        case 1: v1 = o + 1; v2 = o + W; v3 = o + W + WH; break;
        case 2: v1 = o + 1; v2 = o + 1 + W; v3 = o + W + WH; break;
        case 3: v1 = o + 1; v2 = o + WH; v3 = o + W + WH; break;
        case 4: v1 = o + 1; v2 = o + 1 + WH; v3 = o + W + WH; break;
        case 5: v1 = o + 1; v2 = o + W + WH; v3 = o + 1 + W + WH; break;
        default: break;  // negative remainder: the reference leaves the values untouched
        }
    }
    sort_desc3(v1, v2, v3);
    a = v1; b = v2; c = v3;
}

// getVerticesFromTetrahedraID (main_3d.cu:672-740) for any id, sorted descending
__device__ DMTZ_SHARED_CODE void tet_verts(const Grid &g, i64 t, i64 &a, i64 &b, i64 &c, i64 &d) {
    const i64 W = g.W, H = g.H, WH = W * H;
    const i64 base = t / 6;
    const i64 cz = base / ((W - 1) * (H - 1)), cy = (base % ((W - 1) * (H - 1))) / (W - 1), cx = base % (W - 1);
    const i64 o = cx + cy * W + cz * WH;
    i64 v[4] = {0, 0, 0, 0};
    switch (t % 6) {
    case 0: v[0] = o; v[1] = o + 1; v[2] = o + W; v[3] = o + W + WH; break;
    case 1: v[0] = o; v[1] = o + 1; v[2] = o + WH; v[3] = o + W + WH; break;
    case 2: v[0] = o + 1; v[1] = o + W; v[2] = o + 1 + W; v[3] = o + W + WH; break;
    case 3: v[0] = o + 1; v[1] = o + 1 + W; v[2] = o + W + WH; v[3] = o + 1 + W + WH; break;
    case 4: v[0] = o + 1; v[1] = o + WH; v[2] = o + 1 + WH; v[3] = o + W + WH; break;
    case 5: v[0] = o + 1; v[1] = o + 1 + WH; v[2] = o + W + WH; v[3] = o + 1 + W + WH; break;
    default: break;
    }
    // same compare-exchange network as the reference
    i64 tt;
    if (v[0] < v[1]) { tt = v[0]; v[0] = v[1]; v[1] = tt; }
    if (v[0] < v[2]) { tt = v[0]; v[0] = v[2]; v[2] = tt; }
    if (v[0] < v[3]) { tt = v[0]; v[0] = v[3]; v[3] = tt; }
    if (v[1] < v[2]) { tt = v[1]; v[1] = v[2]; v[2] = tt; }
    if (v[1] < v[3]) { tt = v[1]; v[1] = v[3]; v[3] = tt; }
    if (v[2] < v[3]) { tt = v[2]; v[2] = v[3]; v[3] = tt; }
    a = v[0]; b = v[1]; c = v[2]; d = v[3];
}

// --------------------------------------------------------------- pairing accessors
__device__ __forceinline__ i64 edge_ref_pair(const Grid &g, i64 a, i64 b) {
    // edge id of two adjacent vertices
    int ax, ay, az, bx, by, bz;
    decode_v(g, a, ax, ay, az);
    decode_v(g, b, bx, by, bz);
    const int x = min(ax, bx), y = min(ay, by), z = min(az, bz);
    const int ca = (ax - x) + 2 * (ay - y) + 4 * (az - z), cb = (bx - x) + 2 * (by - y) + 4 * (bz - z);
    int k = 0;
    for (int i = 0; i < 7; i++)
        if ((TOPO_EDGE_V[i][0] == ca && TOPO_EDGE_V[i][1] == cb) || (TOPO_EDGE_V[i][0] == cb && TOPO_EDGE_V[i][1] == ca))
            k = i;
    return edge_ref(g, x, y, z, k);
}

// paired_vertices[v]
__device__ DMTZ_SHARED_CODE i64 pv_ref(const RuleCtx &c, const FieldState &s, i64 v) {
    if (v < 0 || v >= c.g.V) {
        atomicOr(c.err, ERR_OOB);
        return -1;
    }
    const int d = s.pv[v];
    if (d == 15) return -1;
    return edge_ref_pair(c.g, v, v + c.g.doff[d]);
}
// paired_edges[e]
__device__ DMTZ_SHARED_CODE i64 pe_ref(const RuleCtx &c, const FieldState &s, i64 e) {
    if (e < 0 || e >= c.g.E) {
        atomicOr(c.err, ERR_OOB);
        return -1;
    }
    int x, y, z, k;
    edge_unref(c.g, e, x, y, z, k);
    const i64 a = x + (i64)y * c.g.W + (i64)z * c.g.WH;
    const int up = eup_get(s.eup[a], k);
    if (up) {
        const signed char *cf = TOPO_EDGE_COF[k][up - 1];
        return face_ref(c.g, x + cf[0], y + cf[1], z + cf[2], cf[3]);
    }
    const int cp = TOPO_EDGE_V[k][0], cq = TOPO_EDGE_V[k][1];
    const i64 p = a + c.g.coff[cp], q = a + c.g.coff[cq];
    if (s.pv[p] == TOPO_CORNER_DIR[cp][cq]) return p;
    if (s.pv[q] == TOPO_CORNER_DIR[cq][cp]) return q;
    return -1;
}
// paired_faces[t]
__device__ DMTZ_SHARED_CODE i64 pf_ref(const RuleCtx &c, const FieldState &s, i64 t) {
    if (t < 0 || t >= c.g.F) {
        atomicOr(c.err, ERR_OOB);
        return -1;
    }
    int x, y, z, sl;
    face_unref(c.g, t, x, y, z, sl);
    const i64 a = x + (i64)y * c.g.W + (i64)z * c.g.WH;
    const int up = fup_get(s.fup[a], sl);
    if (up) {
        const signed char *tc = TOPO_FACE_COF[sl][up - 1];
        return tet_ref(c.g, x + tc[0], y + tc[1], z + tc[2], tc[3]);
    }
    for (int j = 0; j < 3; j++) {
        const signed char *fe = TOPO_FACE_EDGE[sl][j];
        const i64 ea = a + fe[0] + (i64)fe[1] * c.g.W + (i64)fe[2] * c.g.WH;
        if (eup_get(s.eup[ea], fe[3]) == fe[4] + 1) return edge_ref(c.g, x + fe[0], y + fe[1], z + fe[2], fe[3]);
    }
    return -1;
}
// paired_tetrahedras[t]
__device__ DMTZ_SHARED_CODE i64 pt_ref(const RuleCtx &c, const FieldState &s, i64 t) {
    if (t < 0 || t >= c.g.T) {
        atomicOr(c.err, ERR_OOB);
        return -1;
    }
    int x, y, z, sl;
    tet_unref(c.g, t, x, y, z, sl);
    const i64 a = x + (i64)y * c.g.W + (i64)z * c.g.WH;
    for (int j = 0; j < 4; j++) {
        const signed char *tf = TOPO_TET_FACE[sl][j];
        const i64 fa = a + tf[0] + (i64)tf[1] * c.g.W + (i64)tf[2] * c.g.WH;
        if (fup_get(s.fup[fa], tf[3]) == tf[4] + 1) return face_ref(c.g, x + tf[0], y + tf[1], z + tf[2], tf[3]);
    }
    return -1;
}

// --------------------------------------------------------------- values, order, requests
__device__ __forceinline__ double fval(const RuleCtx &c, i64 v) {
    if (v < 0 || v >= c.g.V) {
        atomicOr(c.err, ERR_OOB);
        return 0.0;
    }
    return c.f[v];
}
__device__ __forceinline__ double gval(const RuleCtx &c, i64 v) {
    if (v < 0 || v >= c.g.V) {
        atomicOr(c.err, ERR_OOB);
        return 0.0;
    }
    return c.gv[v];
}
// compare_vertices(a, b, 0|1): (value, id) order
__device__ __forceinline__ bool above_f(const RuleCtx &c, i64 a, i64 b) {
    const uint64_t ka = okey(fval(c, a)), kb = okey(fval(c, b));
    return ka > kb || (ka == kb && a > b);
}
__device__ __forceinline__ bool above_g(const RuleCtx &c, i64 a, i64 b) {
    const uint64_t ka = okey(gval(c, a)), kb = okey(gval(c, b));
    return ka > kb || (ka == kb && a > b);
}
// get_delta (main_3d.cu:239-244)
__device__ __forceinline__ double get_delta(const RuleCtx &c, i64 v) {
    if (v < 0 || v >= c.g.V) {
        atomicOr(c.err, ERR_OOB);
        return 0.0;
    }
    if (c.edit_type == 1) return -ldexp(1.0, -c.cnt[v]) * c.bound;
    return __ddiv_rn(__dsub_rn(__dsub_rn(c.f[v], c.bound), c.gv[v]), 2.0);
}
// "lower v": the reference's swap(v, get_delta(v))
__device__ __forceinline__ void lower(const RuleCtx &c, i64 v) {
    if (v < 0 || v >= c.g.V) {
        atomicOr(c.err, ERR_OOB);
        return;
    }
    const uint32_t bit = 1u << (v & 31);
    const uint32_t old = atomicOr(&c.reqbits[v >> 5], bit);
    if (!(old & bit)) {
        const unsigned long long k = agg_slot(c.reqn);
        if ((i64)k < c.reqcap) c.reqlist[k] = v;
    }
}
__device__ __forceinline__ i64 third_of(i64 a, i64 b, i64 cc, i64 v1, i64 v2) {
    i64 v3 = cc;
    if (a != v1 && a != v2) v3 = a;
    else if (b != v1 && b != v2) v3 = b;
    return v3;
}
__device__ __forceinline__ i64 fourth_of(i64 a, i64 b, i64 cc, i64 d, i64 v1, i64 v2, i64 v3) {
    i64 v4 = d;
    if (a != v1 && a != v2 && a != v3) v4 = a;
    else if (b != v1 && b != v2 && b != v3) v4 = b;
    else if (cc != v1 && cc != v2 && cc != v3) v4 = cc;
    return v4;
}
__device__ __forceinline__ bool adjacent(const Grid &g, i64 a, i64 b, int &d) {
    int ax, ay, az, bx, by, bz;
    decode_v(g, a, ax, ay, az);
    decode_v(g, b, bx, by, bz);
    d = dir_of(bx - ax, by - ay, bz - az);
    return d >= 0;
}

// argmin over the common neighbours n of (v1, v2) with exactly one of v1, v2
// above n in the ORIGINAL field (the rescan of fix_saddle, main_3d.cu:2942-3015)
__device__ DMTZ_SHARED_CODE i64 rescan_edge(const RuleCtx &c, i64 v1, i64 v2) {
    int x1, y1, z1, x2, y2, z2;
    decode_v(c.g, v1, x1, y1, z1);
    decode_v(c.g, v2, x2, y2, z2);
    uint64_t bk = DMTZ_KEY_DBL_MAX;
    i64 bid = INT_MAX;
    bool found = false;
    for (int i = 0; i < 14; i++) {
        const int nx = x1 + TOPO_DIRS[i][0], ny = y1 + TOPO_DIRS[i][1], nz = z1 + TOPO_DIRS[i][2];
        if (!inb(c.g, nx, ny, nz)) continue;
        if (dir_of(nx - x2, ny - y2, nz - z2) < 0) continue;
        const i64 n = nx + (i64)ny * c.g.W + (i64)nz * c.g.WH;
        if (above_f(c, v1, n) != above_f(c, v2, n)) {
            const uint64_t kn = okey(c.f[n]);
            if (kn < bk || (kn == bk && n < bid)) {
                bk = kn;
                bid = n;
                found = true;
            }
        }
    }
    return found ? bid : -1;
}

// get_smallest_vertex (main_3d.cu:2115-2194): common neighbours of a triangle
// below exactly two of its vertices in the ORIGINAL field, argmin
__device__ DMTZ_SHARED_CODE i64 smallest_vertex(const RuleCtx &c, i64 v1, i64 v2, i64 v3) {
    int x1, y1, z1, x2, y2, z2, x3, y3, z3;
    decode_v(c.g, v1, x1, y1, z1);
    decode_v(c.g, v2, x2, y2, z2);
    decode_v(c.g, v3, x3, y3, z3);
    uint64_t bk = DMTZ_KEY_DBL_MAX;
    i64 bid = INT_MAX;
    bool found = false;
    for (int i = 0; i < 14; i++) {
        const int nx = x1 + TOPO_DIRS[i][0], ny = y1 + TOPO_DIRS[i][1], nz = z1 + TOPO_DIRS[i][2];
        if (!inb(c.g, nx, ny, nz)) continue;
        if (dir_of(nx - x2, ny - y2, nz - z2) < 0 || dir_of(nx - x3, ny - y3, nz - z3) < 0) continue;
        const i64 n = nx + (i64)ny * c.g.W + (i64)nz * c.g.WH;
        if (n == v1 || n == v2 || n == v3) continue;
        const bool c1 = above_f(c, v1, n), c2 = above_f(c, v2, n), c3 = above_f(c, v3, n);
        if ((c1 && c2 && !c3) || (c1 && !c2 && c3) || (!c1 && c2 && c3)) {
            const uint64_t kn = okey(c.f[n]);
            if (kn < bk || (kn == bk && n < bid)) {
                bk = kn;
                bid = n;
                found = true;
            }
        }
    }
    return found ? bid : -1;
}

// --------------------------------------------------------------- A8 fix_minimum
__device__ inline void rule_min(const RuleCtx &c, i64 id) {
    const i64 pv = pv_ref(c, c.P, id);
    if (pv != -1) {
        i64 vertex, v2;
        edge_verts(c.g, pv, vertex, v2);
        if (vertex != id) v2 = vertex;
        lower(c, v2);
    } else {
        lower(c, id);
    }
}

// --------------------------------------------------------------- A9 fix_saddle
__device__ inline void rule_saddle(const RuleCtx &c, i64 id) {
    const Grid &G = c.g;
    i64 edge = id;
    const i64 pe = pe_ref(c, c.P, id);
    if (pe != -1) {
        if (pe < G.V && pe >= 0 && pv_ref(c, c.P, pe) == id) {
            i64 v1, v2;
            edge_verts(G, edge, v1, v2);
            if (v2 != pe) v1 = pe;
            else { v2 = v1; v1 = pe; }
            const i64 q = pv_ref(c, c.Q, v1);
            if (q == -1 || q < 0 || q >= G.E) return;
            i64 fv1, fv2;
            edge_verts(G, q, fv1, fv2);
            const i64 false_v2 = v1 == fv1 ? fv2 : fv1;
            const double a = gval(c, v2), b = gval(c, false_v2);
            if (a > b || (a == b && v2 > false_v2)) lower(c, v2);
        } else if (pe < G.F && pe >= 0 && pf_ref(c, c.P, pe) == id) {
            const i64 face = pe;
            i64 v1, v2, a, b, v3;
            edge_verts(G, edge, v1, v2);
            tri_verts(G, face, a, b, v3);
            v3 = third_of(a, b, v3, v1, v2);
            const i64 osv1 = !above_g(c, v1, v3) ? v3 : v1;
            const i64 osv1_1 = !above_g(c, v2, v3) ? v3 : v2;
            const bool v1_edge = above_g(c, v1, v3), v2_edge = above_g(c, v2, v3);
            bool o_v1_edge = above_f(c, v1, v3), o_v2_edge = above_f(c, v2, v3);
            if (v1_edge && v2_edge) {
                lower(c, v3);
            } else if (o_v1_edge && o_v2_edge) {
                lower(c, v3);
            } else {
                const i64 pe2 = pe_ref(c, c.P, id);
                i64 qf = -1;
                bool cond = pe2 != -1 && pe2 < G.F && pe2 >= 0;
                if (cond) {
                    qf = pf_ref(c, c.Q, pe2);
                    cond = qf != -1 && pe_ref(c, c.Q, qf) == pe2;
                }
                if (cond) {
                    const i64 false_edge = qf;
                    edge = false_edge;
                    i64 a1, b1;
                    edge_verts(G, false_edge, a1, b1);
                    const i64 false_v = (a1 != v1 && a1 != v2) ? a1 : b1;
                    const double diff = get_delta(c, false_v);
                    i64 w1, w2, p, q, w3;
                    edge_verts(G, edge, w1, w2);
                    tri_verts(G, face, p, q, w3);
                    w3 = third_of(p, q, w3, w1, w2);
                    o_v1_edge = above_f(c, w2, w3);
                    o_v2_edge = above_f(c, w1, w3);
                    bool take = o_v1_edge && o_v2_edge;
                    i64 pfe = -1;
                    if (take) {
                        pfe = pe_ref(c, c.P, false_edge);
                        take = pfe != -1 && pf_ref(c, c.P, pfe) == false_edge;
                    }
                    if (take) {
                        i64 r, s2, u3;
                        tri_verts(G, pfe, r, s2, u3);
                        u3 = third_of(r, s2, u3, w1, w2);
                        lower(c, u3);
                    } else if (fabs(diff) > 0) {
                        lower(c, false_v);
                    }
                } else {
                    if (o_v1_edge && !v1_edge) lower(c, osv1);
                    else lower(c, osv1_1);
                }
            }
        }
    } else {
        const i64 qe = pe_ref(c, c.Q, id);
        if (qe != -1 && qe < G.V && qe >= 0 && pv_ref(c, c.Q, qe) == id) {
            lower(c, qe);
        } else if (qe != -1 && qe < G.F && qe >= 0 && pf_ref(c, c.Q, qe) == id) {
            i64 v1, v2, a, b, v3;
            edge_verts(G, edge, v1, v2);
            tri_verts(G, qe, a, b, v3);
            v3 = third_of(a, b, v3, v1, v2);
            const bool v1_edge = above_g(c, v2, v3), v2_edge = above_g(c, v1, v3);
            const bool or_v1_edge = above_f(c, v2, v3), or_v2_edge = above_f(c, v1, v3);
            if (v1_edge == v2_edge) {
                if (v1_edge != or_v1_edge) lower(c, v2);
                if (v2_edge != or_v2_edge) lower(c, v1);
            } else {
                // paired_edges[id] is -1 on this branch; the reference's
                // "paired with a vertex" sub-case cannot occur
                const i64 m = rescan_edge(c, v1, v2);
                if (m != -1) {
                    lower(c, m);
                } else {
                    lower(c, v1);
                    lower(c, v2);
                }
            }
        }
    }
}

// --------------------------------------------------------------- A10 fix_2saddle
__device__ inline void rule_2saddle(const RuleCtx &c, i64 id) {
    const Grid &G = c.g;
    const i64 pf = pf_ref(c, c.P, id);
    if (pf != -1) {
        if (pf < G.E && pf >= 0 && pe_ref(c, c.P, pf) == id) {
            const i64 edge = pf;
            i64 v1, v2, a, b, v3;
            edge_verts(G, edge, v1, v2);
            tri_verts(G, id, a, b, v3);
            v3 = third_of(a, b, v3, v1, v2);
            bool v1_edge = above_g(c, v2, v3), v2_edge = above_g(c, v1, v3);
            bool o_v1_edge = above_f(c, v2, v3), o_v2_edge = above_f(c, v1, v3);
            if (v1_edge && v2_edge) {
                const i64 f_id = pe_ref(c, c.P, edge);
                if (f_id == -1 || pf_ref(c, c.P, f_id) != edge) return;
                i64 p, q, w3;
                tri_verts(G, f_id, p, q, w3);
                w3 = third_of(p, q, w3, v1, v2);
                lower(c, w3);
            } else if (o_v1_edge != o_v2_edge && v1_edge != v2_edge) {
                const i64 f_id = pe_ref(c, c.Q, edge);
                if (f_id == -1 || pf_ref(c, c.Q, f_id) != edge) {
                    lower(c, v3);
                } else if (f_id < G.F && f_id >= 0) {
                    i64 p, q, v3_1;
                    tri_verts(G, f_id, p, q, v3_1);
                    v3_1 = third_of(p, q, v3_1, v1, v2);
                    v1_edge = above_g(c, v2, v3_1);
                    v2_edge = above_g(c, v1, v3_1);
                    o_v1_edge = above_f(c, v2, v3_1);
                    o_v2_edge = above_f(c, v1, v3_1);
                    if (v1_edge && v2_edge && ((!o_v1_edge && o_v2_edge) || (o_v1_edge && !o_v2_edge))) {
                        if (!o_v1_edge) lower(c, v2);
                        else lower(c, v1);
                    } else {
                        lower(c, v3);
                    }
                }
            } else if (!above_g(c, v1, v3) || !above_g(c, v2, v3)) {
                lower(c, v3);
            }
        } else if (pf < G.T && pf >= 0 && pt_ref(c, c.P, pf) == id) {
            const i64 tet = pf;
            i64 v1, v2, v3, a, b, cc, v4;
            tri_verts(G, id, v1, v2, v3);
            tet_verts(G, tet, a, b, cc, v4);
            v4 = fourth_of(a, b, cc, v4, v1, v2, v3);
            const bool or1 = above_f(c, v3, v4), or2 = above_f(c, v2, v4), or3 = above_f(c, v1, v4);
            if (!or1 || !or2 || !or3) {
                const i64 pff = pt_ref(c, c.Q, tet);
                if (pff != -1) {
                    i64 v1_1, v2_1, v3_1;
                    tri_verts(G, pff, v1_1, v2_1, v3_1);
                    const bool f1 = above_g(c, v3_1, v4), f2 = above_g(c, v2_1, v4), f3 = above_g(c, v1_1, v4);
                    const bool o1 = above_f(c, v3_1, v4), o2 = above_f(c, v2_1, v4), o3 = above_f(c, v1_1, v4);
                    if ((!f1 || !f2 || !f3) && (!o1 || !o2 || !o3)) {
                        const i64 id2 = pf_ref(c, c.P, pff);
                        if (id2 >= 0 && id2 < G.E && pe_ref(c, c.P, id2) == pff) {
                            i64 w1, w2;
                            edge_verts(G, id2, w1, w2);
                            i64 w3 = v3_1;
                            if (v1_1 != w1 && w2 != v1_1) w3 = v1_1;
                            else if (v2_1 != w1 && v2_1 != w2) w3 = v2_1;
                            lower(c, w3);
                        } else if (id2 >= 0 && id2 < G.T && pt_ref(c, c.P, id2) == pff) {
                            i64 t1, t2, t3, t4;
                            tet_verts(G, id2, t1, t2, t3, t4);
                            if (t1 != v1_1 && t1 != v2_1 && t1 != v3_1) t4 = v1_1;
                            else if (t2 != v1_1 && t2 != v2_1 && t2 != v3_1) t4 = v2_1;
                            else if (t3 != v1_1 && t3 != v2_1 && t3 != v3_1) t4 = v3_1;
                            (void)get_delta(c, t4);
                            lower(c, t1);
                            lower(c, t2);
                            lower(c, t3);
                            lower(c, t4);
                        }
                    } else {
                        lower(c, v1_1);
                        lower(c, v2_1);
                        lower(c, v3_1);
                    }
                } else {
                    lower(c, v4);
                }
            } else {
                lower(c, v4);
            }
        }
    } else {
        const i64 qf = pf_ref(c, c.Q, id);
        if (qf != -1 && qf < G.E && qf >= 0 && pe_ref(c, c.Q, qf) == id) {
            const i64 edge_id = qf;
            i64 v1, v2;
            edge_verts(G, edge_id, v1, v2);
            const i64 sv1 = !above_g(c, v1, v2) ? v2 : v1;
            const i64 sv2 = !above_g(c, v1, v2) ? v1 : v2;
            const i64 true_face_id = pe_ref(c, c.P, edge_id);
            if (true_face_id != -1 && pf_ref(c, c.P, true_face_id) == edge_id) {
                i64 p, q, w3;
                tri_verts(G, true_face_id, p, q, w3);
                if (sv1 != p && sv2 != p) w3 = p;
                if (sv1 != q && sv2 != q) w3 = q;
                lower(c, w3);
            } else if (true_face_id >= 0 && true_face_id < G.V && pv_ref(c, c.P, true_face_id) == edge_id) {
                lower(c, sv1);
                lower(c, sv2);
            }
        } else if (qf != -1 && qf < G.T && qf >= 0 && pt_ref(c, c.Q, qf) == id) {
            const i64 tet = qf;
            i64 v1, v2, v3, a, b, cc, v4;
            tri_verts(G, id, v1, v2, v3);
            tet_verts(G, tet, a, b, cc, v4);
            v4 = fourth_of(a, b, cc, v4, v1, v2, v3);
            const bool f1 = above_g(c, v3, v4), f2 = above_g(c, v2, v4), f3 = above_g(c, v1, v4);
            const bool o1 = above_f(c, v3, v4), o2 = above_f(c, v2, v4), o3 = above_f(c, v1, v4);
            if (f1 && f2 && f3) {
                if (f1 != o1) lower(c, v3);
                else if (f2 != o2) lower(c, v2);
                else if (f3 != o3) lower(c, v1);
            } else {
                const i64 true_cell = pt_ref(c, c.P, tet);
                if (true_cell >= 0 && true_cell < G.T) {
                    lower(c, v1);
                    lower(c, v2);
                    lower(c, v3);
                } else {
                    const i64 m = smallest_vertex(c, v1, v2, v3);
                    if (m != -1) {
                        lower(c, m);
                    } else {
                        lower(c, v1);
                        lower(c, v2);
                        lower(c, v3);
                    }
                }
            }
        }
    }
}

// --------------------------------------------------------------- A11 fix_maximum
__device__ inline void rule_max(const RuleCtx &c, i64 id) {
    const Grid &G = c.g;
    const i64 pt = pt_ref(c, c.P, id);
    if (pt != -1) {
        const i64 face1 = pt;
        i64 v1, v2, v3, a, b, cc, v4;
        tri_verts(G, face1, v1, v2, v3);
        tet_verts(G, id, a, b, cc, v4);
        v4 = fourth_of(a, b, cc, v4, v1, v2, v3);
        const bool o1 = above_f(c, v1, v4), o2 = above_f(c, v2, v4), o3 = above_f(c, v3, v4);
        if (o1 && o2 && o3) {
            lower(c, v4);
        } else {
            const i64 fc = pf_ref(c, c.Q, face1);
            if (fc >= 0) {
                if (fc < G.E && pe_ref(c, c.Q, fc) == face1) {
                    i64 e1, e2;
                    edge_verts(G, fc, e1, e2);
                    lower(c, above_g(c, e1, e2) ? e1 : e2);
                } else if (fc < G.T && pt_ref(c, c.Q, fc) == face1) {
                    lower(c, v4);
                }
            }
        }
    } else {
        const i64 face1 = pt_ref(c, c.Q, id);
        i64 v1, v2, v3, a, b, cc, v4;
        tri_verts(G, face1, v1, v2, v3);
        tet_verts(G, id, a, b, cc, v4);
        v4 = fourth_of(a, b, cc, v4, v1, v2, v3);
        const bool f1 = above_g(c, v1, v4), f2 = above_g(c, v2, v4), f3 = above_g(c, v3, v4);
        const bool o1 = above_f(c, v1, v4), o2 = above_f(c, v2, v4), o3 = above_f(c, v3, v4);
        if (f1 && f2 && f3) {
            if (!o1 && f1) lower(c, v1);
            if (!o2 && f2) lower(c, v2);
            if (!o3 && f3) lower(c, v3);
            if (o1 && o2 && o3) {
                const i64 it = pf_ref(c, c.P, face1);
                if (it != -1) {
                    // the reference reads this id as a tetrahedron whatever its kind
                    if (it < 0 || it >= G.T) atomicOr(c.err, ERR_OOB);
                    i64 p, q, r, w4;
                    tet_verts(G, it, p, q, r, w4);
                    w4 = fourth_of(p, q, r, w4, v1, v2, v3);
                    lower(c, w4);
                }
            }
        } else {
            const i64 pid = pf_ref(c, c.P, face1);
            if (pid != -1) {
                if (pid >= 0 && pid < G.E && pe_ref(c, c.P, pid) == face1) {
                    i64 e1, e2;
                    edge_verts(G, pid, e1, e2);
                    lower(c, e1);
                    lower(c, e2);
                } else {
                    if (pid < 0 || pid >= G.T) atomicOr(c.err, ERR_OOB);
                    i64 p, q, r, s2;
                    tet_verts(G, pid, p, q, r, s2);
                    lower(c, p);
                    lower(c, q);
                    lower(c, r);
                    lower(c, s2);
                }
            } else {
                if (!o1) lower(c, v1);
                if (!o2) lower(c, v2);
                if (!o3) lower(c, v3);
            }
        }
    }
}

// --------------------------------------------------------------- A12/A13 separatrix checks
// cofaces of a triangle in get_cell_tetra order (main_3d.cu:4363-4430):
// x = first existing coface, y = last existing (left as given when only one)
__device__ inline int face_cofaces(const Grid &g, i64 t, i64 out[2]) {
    int x, y, z, sl;
    face_unref(g, t, x, y, z, sl);
    int n = 0;
    for (int j = 0; j < TOPO_FACE_NCOF[sl]; j++) {
        const signed char *tc = TOPO_FACE_COF[sl][j];
        if (!cell_ok(g, x + tc[0], y + tc[1], z + tc[2], 1, 1, 1)) continue;
        out[n++] = tet_ref(g, x + tc[0], y + tc[1], z + tc[2], tc[3]);
    }
    return n;
}

// --------------------------------------------------------------- A15 fix_as_vpath (type 2)
__device__ inline void rule_as_path(const RuleCtx &c, i64 t_idx) {
    const Grid &G = c.g;
    const i64 true_edge = pt_ref(c, c.P, t_idx);
    const i64 false_edge = pt_ref(c, c.Q, t_idx);
    const i64 pfe = pf_ref(c, c.P, false_edge);
    if (pfe >= 0 && pfe < G.T && pt_ref(c, c.P, pfe) == false_edge) {
        i64 v1, v2, v3, a, b, cc, d;
        tri_verts(G, false_edge, v1, v2, v3);
        tet_verts(G, pfe, a, b, cc, d);
        lower(c, fourth_of(a, b, cc, d, v1, v2, v3));
    } else {
        i64 v1, v2, v3, a, b, tv3;
        tri_verts(G, true_edge, v1, v2, v3);
        tri_verts(G, false_edge, a, b, tv3);
        if (a != v1 && a != v2 && a != v3) tv3 = a;
        else if (b != v1 && b != v2 && b != v3) tv3 = b;
        lower(c, tv3);
    }
}
// A14 fix_ds_vpath (type 0)
__device__ inline void rule_ds_path(const RuleCtx &c, i64 v_idx) {
    const i64 tpe = pv_ref(c, c.P, v_idx);
    i64 v1, v2;
    edge_verts(c.g, tpe, v1, v2);
    lower(c, v_idx == v1 ? v2 : v1);
}

// fix_ds_wall (main_3d.cu:5297-5413) for the wall record edge e: the edge's
// original and decompressed pairings differ
__device__ inline void rule_ds_wall(const RuleCtx &c, i64 e) {
    const Grid &G = c.g;
    const i64 tf = pe_ref(c, c.P, e), ff = pe_ref(c, c.Q, e);
    if (tf == ff) return;
    i64 v1, v2;
    edge_verts(G, e, v1, v2);
    if (tf >= 0 && ff >= 0 && tf < G.F && pf_ref(c, c.P, tf) == e && ff < G.F && pf_ref(c, c.Q, ff) == e) {
        // both pair the edge with a face: lower the original face's third vertex,
        // or both endpoints when that vertex has no room left
        i64 a, b, v3;
        tri_verts(G, tf, a, b, v3);
        if (a != v1 && a != v2) v3 = a;
        if (b != v1 && b != v2) v3 = b;
        if (fabs(get_delta(c, v3)) > 1e-16 * c.range) {
            lower(c, v3);
        } else {
            lower(c, v1);
            lower(c, v2);
        }
    } else if (tf == -1 || tf >= G.F || (tf >= 0 && pf_ref(c, c.P, tf) != e)) {
        lower(c, v1);
        lower(c, v2);
    } else if (ff == -1 || ff >= G.F || (ff >= 0 && pf_ref(c, c.Q, ff) != e)) {
        i64 a, b, v3;
        tri_verts(G, tf, a, b, v3);
        lower(c, third_of(a, b, v3, v1, v2));
    }
}

}  // namespace dmtz
