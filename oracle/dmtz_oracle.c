/*
 * dmtz_oracle.c — CPU oracle (test infrastructure only) for the DMTz
 * topology-correction path.  A serial restatement of the reference kernels in
 * main_3d.cu; every function names the lines it follows.  The product library
 * never links or calls this file: tests, the smoke check and bench.py's CPU
 * baseline leg use it as the checker.
 *
 * Semantics are kept literal, including the reference's quirks (shadowed
 * variables, if/if chains, union-valued pairing arrays disambiguated by
 * back-pointer checks, guarded writes of the delta buffer).  Index
 * arithmetic on invalid ids reproduces the reference's integer arithmetic;
 * every array access outside its allocation is counted in `oob` instead of
 * being performed, so a caller can tell when the reference itself would have
 * read or written out of bounds (parity is then void for that input).
 */
#include "dmtz_oracle.h"

#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Freudenthal 1-ring stencil, same order as directions1 (main_3d.cu:44-51) */
static const int DIRS[14][3] = {
    {1, 0, 0},  {-1, 0, 0}, {0, 1, 0},  {0, -1, 0}, {0, 0, 1},
    {0, 0, -1}, {-1, 1, 0}, {1, -1, 0}, {0, 1, 1},  {0, -1, -1},
    {-1, 0, 1}, {1, 0, -1}, {-1, 1, 1}, {1, -1, -1}};

/* 3x3x3 membership table of the stencil, indexed by (dx+1) + 3(dy+1) + 9(dz+1) */
static const unsigned char DIR_LUT[27] = {0, 1, 1, 0, 1, 1, 0, 0, 0, 0, 1, 1, 1, 0,
                                          1, 1, 1, 0, 0, 0, 0, 1, 1, 0, 1, 1, 0};

static int is_dir(int dx, int dy, int dz) {
    if (dx < -1 || dx > 1 || dy < -1 || dy > 1 || dz < -1 || dz > 1) return 0;
    return DIR_LUT[(dx + 1) + 3 * (dy + 1) + 9 * (dz + 1)];
}

typedef struct {
    int W, H, D;
    int V, E, F, T;
} grid_t;

static void grid_init(grid_t *G, int W, int H, int D) {
    G->W = W;
    G->H = H;
    G->D = D;
    G->V = W * H * D;
    /* main_3d.cu:6403-6415 */
    G->E = (W - 1) * H * D + W * (H - 1) * D + W * H * (D - 1) + (W - 1) * (H - 1) * D +
           (W - 1) * H * (D - 1) + W * (H - 1) * (D - 1) + (W - 1) * (H - 1) * (D - 1);
    G->F = 2 * ((W - 1) * (H - 1) * D + W * (H - 1) * (D - 1) + (W - 1) * H * (D - 1)) +
           6 * (W - 1) * (H - 1) * (D - 1);
    G->T = 6 * (W - 1) * (H - 1) * (D - 1);
}

void orc_counts(int W, int H, int D, long long out[4]) {
    grid_t G;
    grid_init(&G, W, H, D);
    out[0] = G.V;
    out[1] = G.E;
    out[2] = G.F;
    out[3] = G.T;
}

#define SWAPI(a, b)   \
    do {              \
        int t_ = (a); \
        (a) = (b);    \
        (b) = t_;     \
    } while (0)

/* ---------------------------------------------------------------------------
 * A0: id <-> vertex tuples
 * ------------------------------------------------------------------------- */

/* getEdgeID, main_3d.cu:917-1012 */
static int edge_id(const grid_t *G, int x, int y, int z, int x1, int y1, int z1) {
    const int W = G->W, H = G->H, D = G->D;
    const int dx = x1 - x, dy = y1 - y, dz = z1 - z;
    const int o1 = (W - 1) * H * D;
    const int o2 = o1 + W * (H - 1) * D;
    const int o3 = o2 + W * H * (D - 1);
    const int o4 = o3 + (W - 1) * (H - 1) * D;
    const int o5 = o4 + W * (H - 1) * (D - 1);
    const int o6 = o5 + (W - 1) * H * (D - 1);
    if (dx == 1 && dy == 0 && dz == 0) return z * (W - 1) * H + y * (W - 1) + x;
    if (dx == -1 && dy == 0 && dz == 0) return z * (W - 1) * H + y * (W - 1) + (x - 1);
    if (dx == 0 && dy == 1 && dz == 0) return o1 + z * W * (H - 1) + x * (H - 1) + y;
    if (dx == 0 && dy == -1 && dz == 0) return o1 + z * W * (H - 1) + x * (H - 1) + y - 1;
    if (dx == 0 && dy == 0 && dz == 1) return o2 + y * W * (D - 1) + x * (D - 1) + z;
    if (dx == 0 && dy == 0 && dz == -1) return o2 + y * W * (D - 1) + x * (D - 1) + z - 1;
    if (dx == 1 && dy == -1 && dz == 0) return o3 + z * (H - 1) * (W - 1) + (y - 1) * (W - 1) + x;
    if (dx == -1 && dy == 1 && dz == 0) return o3 + z * (H - 1) * (W - 1) + y * (W - 1) + (x - 1);
    if (dx == 0 && dy == 1 && dz == 1) return o4 + x * (H - 1) * (D - 1) + y * (D - 1) + z;
    if (dx == 0 && dy == -1 && dz == -1) return o4 + x * (H - 1) * (D - 1) + (y - 1) * (D - 1) + z - 1;
    if (dx == -1 && dy == 0 && dz == 1) return o5 + y * (W - 1) * (D - 1) + z * (W - 1) + x - 1;
    if (dx == 1 && dy == 0 && dz == -1) return o5 + y * (W - 1) * (D - 1) + (z - 1) * (W - 1) + x;
    if (dx != 0 && dy != 0 && dz != 0) {
        int cx = x < x1 ? x : x1, cy = y < y1 ? y : y1, cz = z < z1 ? z : z1;
        return o6 + cz * (W - 1) * (H - 1) + cy * (W - 1) + cx;
    }
    return -1;
}

/* getVertexIDsFromEdgeID, main_3d.cu:1760-1900; *a > *b */
static void edge_verts(const grid_t *G, int e, int *a, int *b) {
    const int W = G->W, H = G->H, D = G->D;
    int counts[7] = {(W - 1) * H * D,       W * (H - 1) * D,           W * H * (D - 1),
                     (W - 1) * (H - 1) * D, W * (H - 1) * (D - 1),     (W - 1) * H * (D - 1),
                     (W - 1) * (H - 1) * (D - 1)};
    int acc = 0, k = -1;
    for (int i = 0; i < 7; i++) {
        if (e < acc + counts[i]) {
            k = i;
            break;
        }
        acc += counts[i];
    }
    if (k == -1) {
        *a = *b = -1;
        return;
    }
    int r = e - acc;
    int x = 0, y = 0, z = 0, x1 = 0, y1 = 0, z1 = 0;
    switch (k) {
    case 0:
        z = r / ((W - 1) * H);
        y = (r % ((W - 1) * H)) / (W - 1);
        x = r % (W - 1);
        x1 = x + 1; y1 = y; z1 = z;
        break;
    case 1:
        z = r / (W * (H - 1));
        x = (r % (W * (H - 1))) / (H - 1);
        y = r % (H - 1);
        y1 = y + 1; x1 = x; z1 = z;
        break;
    case 2:
        y = r / (W * (D - 1));
        x = (r % (W * (D - 1))) / (D - 1);
        z = r % (D - 1);
        y1 = y; x1 = x; z1 = z + 1;
        break;
    case 3: {
        int z2 = r / ((W - 1) * (H - 1));
        int y2 = (r % ((W - 1) * (H - 1))) / (W - 1);
        int x2 = r % (W - 1);
        x = x2 + 1; y = y2; z = z2;
        y1 = y2 + 1; x1 = x2; z1 = z2;
    } break;
    case 4: {
        int x2 = r / ((H - 1) * (D - 1));
        int y2 = (r % ((H - 1) * (D - 1))) / (D - 1);
        int z2 = r % (D - 1);
        x = x2; y = y2; z = z2;
        y1 = y2 + 1; x1 = x2; z1 = z2 + 1;
    } break;
    case 5: {
        int y2 = r / ((W - 1) * (D - 1));
        int z2 = (r % ((W - 1) * (D - 1))) / (W - 1);
        int x2 = r % (W - 1);
        x = x2 + 1; y = y2; z = z2;
        y1 = y2; x1 = x2; z1 = z2 + 1;
    } break;
    default: {
        int z2 = r / ((W - 1) * (H - 1));
        int y2 = (r % ((W - 1) * (H - 1))) / (W - 1);
        int x2 = r % (W - 1);
        x = x2 + 1; y = y2; z = z2;
        y1 = y2 + 1; x1 = x2; z1 = z2 + 1;
    } break;
    }
    int id1 = x + y * W + z * (W * H);
    int id2 = x1 + y1 * W + z1 * (W * H);
    if (id1 < id2) SWAPI(id1, id2);
    *a = id1;
    *b = id2;
}

static void sort3_desc(int *a, int *b, int *c) {
    if (*a < *b) SWAPI(*a, *b);
    if (*a < *c) SWAPI(*a, *c);
    if (*b < *c) SWAPI(*b, *c);
}

/* getTriangleID / getTriangleID1, main_3d.cu:246-423 */
static int tri_id(const grid_t *G, int v1, int v2, int v3) {
    const int W = G->W, H = G->H, D = G->D;
    int s1 = v1, s2 = v2, s3 = v3;
    sort3_desc(&s1, &s2, &s3);
    int x1 = s1 % W, y1 = (s1 / W) % H, z1 = (s1 / (W * H)) % D;
    int x2 = s2 % W, y2 = (s2 / W) % H, z2 = (s2 / (W * H)) % D;
    int x3 = s3 % W, y3 = (s3 / W) % H, z3 = (s3 / (W * H)) % D;
    int mx = x1 < x2 ? x1 : x2; mx = mx < x3 ? mx : x3;
    int my = y1 < y2 ? y1 : y2; my = my < y3 ? my : y3;
    int mz = z1 < z2 ? z1 : z2; mz = mz < z3 ? mz : z3;
    const int bxy = 2 * D * (W - 1) * (H - 1);
    const int byz = bxy + 2 * W * (H - 1) * (D - 1);
    const int bxz = byz + 2 * H * (W - 1) * (D - 1);
    if (z1 == z2 && z2 == z3) { /* xy plane */
        int cell = my * (W - 1) + mx;
        if (x3 == x1 && x1 == mx && y3 == y2 && y2 == my) return cell * 2 + 2 * mz * (W - 1) * (H - 1);
        return cell * 2 + 1 + 2 * mz * (W - 1) * (H - 1);
    }
    if (x1 == x2 && x2 == x3) { /* yz plane */
        int cell = my * (D - 1) + mz;
        if (y2 == y1 && y1 == my + 1 && z3 == z2 && z2 == mz)
            return cell * 2 + bxy + 2 * mx * (H - 1) * (D - 1);
        return cell * 2 + 1 + bxy + 2 * mx * (H - 1) * (D - 1);
    }
    if (y1 == y2 && y2 == y3) { /* xz plane */
        int cell = mz * (W - 1) + mx;
        if (z2 == z3 && z2 == mz && x1 == x3 && x1 == mx)
            return cell * 2 + 2 * (D * (W - 1) * (H - 1) + W * (H - 1) * (D - 1) + my * (W - 1) * (D - 1));
        return cell * 2 + 1 + 2 * (D * (W - 1) * (H - 1) + W * (H - 1) * (D - 1) + my * (W - 1) * (D - 1));
    }
    /* interior */
    int cell = mz * (W - 1) * (H - 1) + my * (W - 1) + mx;
    int cur = -1;
#define P3(X3, Y3, Z3, X2, Y2, Z2, X1, Y1, Z1)                                                                \
    (x3 == mx + (X3) && y3 == my + (Y3) && z3 == mz + (Z3) && x2 == mx + (X2) && y2 == my + (Y2) &&         \
     z2 == mz + (Z2) && x1 == mx + (X1) && y1 == my + (Y1) && z1 == mz + (Z1))
    if (P3(0, 0, 0, 1, 0, 0, 0, 1, 1)) cur = 0;
    if (P3(1, 0, 0, 0, 1, 0, 0, 1, 1)) cur = 1;
    if (P3(1, 0, 0, 1, 1, 0, 0, 1, 1)) cur = 2;
    if (P3(1, 0, 0, 0, 0, 1, 0, 1, 1)) cur = 3;
    if (P3(1, 0, 0, 1, 0, 1, 0, 1, 1)) cur = 4;
    if (P3(1, 0, 0, 0, 1, 1, 1, 1, 1)) cur = 5;
#undef P3
    return cell * 6 + cur + bxz;
}

/* getVerticesFromTriangleID, main_3d.cu:425-565; sorted descending */
static void tri_verts(const grid_t *G, int t, int *a, int *b, int *c) {
    const int W = G->W, H = G->H, D = G->D;
    int base, mx, my, mz, v1 = 0, v2 = 0, v3 = 0;
    const int WH = W * H;
    if (t < 2 * D * (W - 1) * (H - 1)) {
        base = t / 2;
        mz = base / ((W - 1) * (H - 1));
        my = (base % ((W - 1) * (H - 1))) / (W - 1);
        mx = base % (W - 1);
        if (t % 2 == 0) {
            v1 = mx + my * W + mz * WH;
            v2 = (mx + 1) + my * W + mz * WH;
            v3 = mx + (my + 1) * W + mz * WH;
        } else {
            v1 = (mx + 1) + (my + 1) * W + mz * WH;
            v2 = (mx + 1) + my * W + mz * WH;
            v3 = mx + (my + 1) * W + mz * WH;
        }
        sort3_desc(&v1, &v2, &v3);
        *a = v1; *b = v2; *c = v3;
        return;
    }
    t -= 2 * D * (W - 1) * (H - 1);
    if (t < 2 * W * (H - 1) * (D - 1)) {
        base = t / 2;
        mx = base / ((H - 1) * (D - 1));
        my = (base % ((H - 1) * (D - 1))) / (D - 1);
        mz = base % (D - 1);
        if (t % 2 == 0) {
            v1 = mx + my * W + mz * WH;
            v2 = mx + (my + 1) * W + mz * WH;
            v3 = mx + (my + 1) * W + (mz + 1) * WH;
        } else {
            v1 = mx + my * W + mz * WH;
            v2 = mx + my * W + (mz + 1) * WH;
            v3 = mx + (my + 1) * W + (mz + 1) * WH;
        }
        sort3_desc(&v1, &v2, &v3);
        *a = v1; *b = v2; *c = v3;
        return;
    }
    t -= 2 * W * (H - 1) * (D - 1);
    if (t < 2 * H * (W - 1) * (D - 1)) {
        base = t / 2;
        my = base / ((W - 1) * (D - 1));
        mz = (base % ((W - 1) * (D - 1))) / (W - 1);
        mx = base % (W - 1);
        if (t % 2 == 0) {
            v1 = mx + my * W + mz * WH;
            v2 = (mx + 1) + my * W + mz * WH;
            v3 = mx + my * W + (mz + 1) * WH;
        } else {
            v1 = (mx + 1) + my * W + mz * WH;
            v2 = mx + my * W + (mz + 1) * WH;
            v3 = (mx + 1) + my * W + (mz + 1) * WH;
        }
        sort3_desc(&v1, &v2, &v3);
        *a = v1; *b = v2; *c = v3;
        return;
    }
    t -= 2 * H * (W - 1) * (D - 1);
    base = t / 6;
    mz = base / ((W - 1) * (H - 1));
    my = (base % ((W - 1) * (H - 1))) / (W - 1);
    mx = base % (W - 1);
    switch (t % 6) {
    case 0:
        v1 = mx + my * W + mz * WH;
        v2 = mx + 1 + my * W + mz * WH;
        v3 = mx + (my + 1) * W + (mz + 1) * WH;
        break;
    case 1:
        v1 = (mx + 1) + my * W + mz * WH;
        v2 = mx + (my + 1) * W + mz * WH;
        v3 = mx + (my + 1) * W + (mz + 1) * WH;
        break;
    case 2:
        v1 = mx + 1 + my * W + mz * WH;
        v2 = (mx + 1) + (my + 1) * W + mz * WH;
        v3 = mx + (my + 1) * W + (mz + 1) * WH;
        break;
    case 3:
        v1 = (mx + 1) + my * W + mz * WH;
        v2 = mx + my * W + (mz + 1) * WH;
        v3 = mx + (my + 1) * W + (mz + 1) * WH;
        break;
    case 4:
        v1 = (mx + 1) + my * W + mz * WH;
        v2 = (mx + 1) + my * W + (mz + 1) * WH;
        v3 = mx + (my + 1) * W + (mz + 1) * WH;
        break;
    case 5:
        v1 = (mx + 1) + my * W + mz * WH;
        v2 = mx + (my + 1) * W + (mz + 1) * WH;
        v3 = (mx + 1) + (my + 1) * W + (mz + 1) * WH;
        break;
    default: /* negative remainder: the reference's switch leaves v1..v3 untouched */
        break;
    }
    sort3_desc(&v1, &v2, &v3);
    *a = v1; *b = v2; *c = v3;
}

/* getTetrahedraID, main_3d.cu:572-670 */
static int tet_id(const grid_t *G, int v1, int v2, int v3, int v4) {
    const int W = G->W, H = G->H, D = G->D;
#define MIN2(p, q) ((p) < (q) ? (p) : (q))
    int mx = MIN2(MIN2(v1 % W, v2 % W), MIN2(v3 % W, v4 % W));
    int my = MIN2(MIN2((v1 / W) % H, (v2 / W) % H), MIN2((v3 / W) % H, (v4 / W) % H));
    int mz = MIN2(MIN2((v1 / (W * H)) % D, (v2 / (W * H)) % D), MIN2((v3 / (W * H)) % D, (v4 / (W * H)) % D));
#undef MIN2
    int cell = mz * (W - 1) * (H - 1) + my * (W - 1) + mx;
    int s1 = v1, s2 = v2, s3 = v3, s4 = v4;
    if (s1 < s2) SWAPI(s1, s2);
    if (s1 < s3) SWAPI(s1, s3);
    if (s1 < s4) SWAPI(s1, s4);
    if (s2 < s3) SWAPI(s2, s3);
    if (s2 < s4) SWAPI(s2, s4);
    if (s3 < s4) SWAPI(s3, s4);
    int x1 = s1 % W, y1 = (s1 / W) % H, z1 = (s1 / (W * H)) % D;
    int x2 = s2 % W, y2 = (s2 / W) % H, z2 = (s2 / (W * H)) % D;
    int x3 = s3 % W, y3 = (s3 / W) % H, z3 = (s3 / (W * H)) % D;
    int x4 = s4 % W, y4 = (s4 / W) % H, z4 = (s4 / (W * H)) % D;
#define P4(X4, Y4, Z4, X3, Y3, Z3, X2, Y2, Z2, X1, Y1, Z1)                                                  \
    (x4 == mx + (X4) && y4 == my + (Y4) && z4 == mz + (Z4) && x3 == mx + (X3) && y3 == my + (Y3) &&         \
     z3 == mz + (Z3) && x2 == mx + (X2) && y2 == my + (Y2) && z2 == mz + (Z2) && x1 == mx + (X1) &&         \
     y1 == my + (Y1) && z1 == mz + (Z1))
    if (P4(0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 1, 1)) return cell * 6;
    if (P4(0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 1, 1)) return cell * 6 + 1;
    if (P4(1, 0, 0, 0, 1, 0, 1, 1, 0, 0, 1, 1)) return cell * 6 + 2;
    if (P4(1, 0, 0, 1, 1, 0, 0, 1, 1, 1, 1, 1)) return cell * 6 + 3;
    if (P4(1, 0, 0, 0, 0, 1, 1, 0, 1, 0, 1, 1)) return cell * 6 + 4;
    if (P4(1, 0, 0, 1, 0, 1, 0, 1, 1, 1, 1, 1)) return cell * 6 + 5;
#undef P4
    return -1;
}

/* getVerticesFromTetrahedraID, main_3d.cu:672-740; sorted descending */
static void tet_verts(const grid_t *G, int t, int *a, int *b, int *c, int *d) {
    const int W = G->W, H = G->H;
    const int WH = W * H;
    int base = t / 6, type = t % 6;
    int cz = base / ((W - 1) * (H - 1));
    int cy = (base % ((W - 1) * (H - 1))) / (W - 1);
    int cx = base % (W - 1);
    int v1 = 0, v2 = 0, v3 = 0, v4 = 0;
    switch (type) {
    case 0:
        v1 = cx + cy * W + cz * WH;
        v2 = cx + 1 + cy * W + cz * WH;
        v3 = cx + (cy + 1) * W + cz * WH;
        v4 = cx + (cy + 1) * W + (cz + 1) * WH;
        break;
    case 1:
        v1 = cx + cy * W + cz * WH;
        v2 = (cx + 1) + cy * W + cz * WH;
        v3 = cx + cy * W + (cz + 1) * WH;
        v4 = cx + (cy + 1) * W + (cz + 1) * WH;
        break;
    case 2:
        v1 = (cx + 1) + cy * W + cz * WH;
        v2 = cx + (cy + 1) * W + cz * WH;
        v3 = (cx + 1) + (cy + 1) * W + cz * WH;
        v4 = cx + (cy + 1) * W + (cz + 1) * WH;
        break;
    case 3:
        v1 = (cx + 1) + cy * W + cz * WH;
        v2 = (cx + 1) + (cy + 1) * W + cz * WH;
        v3 = cx + (cy + 1) * W + (cz + 1) * WH;
        v4 = (cx + 1) + (cy + 1) * W + (cz + 1) * WH;
        break;
    case 4:
        v1 = (cx + 1) + cy * W + cz * WH;
        v2 = cx + cy * W + (cz + 1) * WH;
        v3 = (cx + 1) + cy * W + (cz + 1) * WH;
        v4 = cx + (cy + 1) * W + (cz + 1) * WH;
        break;
    case 5:
        v1 = (cx + 1) + cy * W + cz * WH;
        v2 = (cx + 1) + cy * W + (cz + 1) * WH;
        v3 = cx + (cy + 1) * W + (cz + 1) * WH;
        v4 = (cx + 1) + (cy + 1) * W + (cz + 1) * WH;
        break;
    default:
        break;
    }
    if (v1 < v2) SWAPI(v1, v2);
    if (v1 < v3) SWAPI(v1, v3);
    if (v1 < v4) SWAPI(v1, v4);
    if (v2 < v3) SWAPI(v2, v3);
    if (v2 < v4) SWAPI(v2, v4);
    if (v3 < v4) SWAPI(v3, v4);
    *a = v1; *b = v2; *c = v3; *d = v4;
}

/* ---------------------------------------------------------------------------
 * Bounds-checked context for the detection and fix rules
 * ------------------------------------------------------------------------- */
typedef struct {
    grid_t G;
    const double *f, *g;
    const int *PV, *PE, *PF, *PT;
    const int *QV, *QE, *QF, *QT;
    const int *cnt;
    double bound, range, sentinel;
    int edit_type;
    double *buf;
    int oob;
} ctx_t;

static int rd(ctx_t *c, const int *a, int n, int i) {
    if (i < 0 || i >= n) {
        c->oob++;
        return -1;
    }
    return a[i];
}
#define PVa(i) rd(c, c->PV, c->G.V, (i))
#define PEa(i) rd(c, c->PE, c->G.E, (i))
#define PFa(i) rd(c, c->PF, c->G.F, (i))
#define PTa(i) rd(c, c->PT, c->G.T, (i))
#define QVa(i) rd(c, c->QV, c->G.V, (i))
#define QEa(i) rd(c, c->QE, c->G.E, (i))
#define QFa(i) rd(c, c->QF, c->G.F, (i))
#define QTa(i) rd(c, c->QT, c->G.T, (i))

static double fv(ctx_t *c, int v) {
    if (v < 0 || v >= c->G.V) {
        c->oob++;
        return 0.0;
    }
    return c->f[v];
}
static double gv(ctx_t *c, int v) {
    if (v < 0 || v >= c->G.V) {
        c->oob++;
        return 0.0;
    }
    return c->g[v];
}

/* compare_vertices, main_3d.cu:1043-1049 (type 0 = original, 1 = decompressed) */
static int above_f(ctx_t *c, int a, int b) {
    double x = fv(c, a), y = fv(c, b);
    return x > y || (x == y && a > b);
}
static int above_g(ctx_t *c, int a, int b) {
    double x = gv(c, a), y = gv(c, b);
    return x > y || (x == y && a > b);
}

/* get_delta, main_3d.cu:239-244 */
static double get_delta(ctx_t *c, int v) {
    if (v < 0 || v >= c->G.V) {
        c->oob++;
        return 0.0;
    }
    if (c->edit_type == 1) return -ldexp(1.0, -c->cnt[v]) * c->bound;
    return (c->f[v] - c->bound - c->g[v]) / 2.0;
}

/* swap / swap1, main_3d.cu:1088-1120: atomic max (edit_type 0) or store */
static void swap_d(ctx_t *c, int v, double diff) {
    if (v < 0 || v >= c->G.V) {
        c->oob++;
        return;
    }
    if (c->edit_type == 0) {
        if (diff > c->buf[v]) c->buf[v] = diff;
    } else {
        c->buf[v] = diff;
    }
}
/* the common call pattern "diff = get_delta(v); swap(v, diff)" */
static void lower(ctx_t *c, int v) { swap_d(c, v, get_delta(c, v)); }
/* the guarded pattern "if (diff > d_deltaBuffer[v]) swap(v, diff)" */
static void lower_guarded(ctx_t *c, int v) {
    double diff = get_delta(c, v);
    if (v < 0 || v >= c->G.V) {
        c->oob++;
        return;
    }
    if (diff > c->buf[v]) swap_d(c, v, diff);
}

/* the vertex of face (a,b,c) that is not an endpoint of edge (v1,v2), with the
 * reference's "if / else if" fallback to the last one */
static int third_of(int a, int b, int cc, int v1, int v2) {
    int v3 = cc;
    if (a != v1 && a != v2) v3 = a;
    else if (b != v1 && b != v2) v3 = b;
    return v3;
}
/* the vertex of tet (a,b,c,d) not in face (v1,v2,v3), reference fallback */
static int fourth_of(int a, int b, int cc, int d, int v1, int v2, int v3) {
    int v4 = d;
    if (a != v1 && a != v2 && a != v3) v4 = a;
    else if (b != v1 && b != v2 && b != v3) v4 = b;
    else if (cc != v1 && cc != v2 && cc != v3) v4 = cc;
    return v4;
}

static void coords(const grid_t *G, int v, int *x, int *y, int *z) {
    *x = v % G->W;
    *y = (v / G->W) % G->H;
    *z = (v / (G->W * G->H)) % G->D;
}

/* get_smallest_vertex, main_3d.cu:2115-2194 (uses the ORIGINAL field) */
static int smallest_vertex(ctx_t *c, int v1, int v2, int v3) {
    const grid_t *G = &c->G;
    int x1, y1, z1, x2, y2, z2, x3, y3, z3;
    coords(G, v1, &x1, &y1, &z1);
    coords(G, v2, &x2, &y2, &z2);
    coords(G, v3, &x3, &y3, &z3);
    int gid = INT_MAX, pid = -1;
    double best = DBL_MAX;
    for (int i = 0; i < 14; i++) {
        int nx = x1 + DIRS[i][0], ny = y1 + DIRS[i][1], nz = z1 + DIRS[i][2];
        int n = nx + ny * G->W + nz * G->W * G->H;
        if (nx >= G->W || ny >= G->H || nz >= G->D || nx < 0 || ny < 0 || nz < 0 || n >= G->V || n < 0) continue;
        if (!is_dir(nx - x2, ny - y2, nz - z2) || !is_dir(nx - x3, ny - y3, nz - z3)) continue;
        if (n == v1 || n == v2 || n == v3) continue;
        int tid = tet_id(G, v1, v2, v3, n);
        int c1 = above_f(c, v1, n), c2 = above_f(c, v2, n), c3 = above_f(c, v3, n);
        if ((c1 && c2 && !c3) || (c1 && !c2 && c3) || (!c1 && c2 && c3)) {
            double fn = fv(c, n);
            if (fn < best || (fn == best && n < gid)) {
                best = fn;
                gid = n;
                pid = tid;
            }
        }
    }
    return pid != -1 ? gid : -1;
}

/* ---------------------------------------------------------------------------
 * A1-A5: discrete gradient (processVertices, edgePairingKernel,
 * trianglePairingKernel), main_3d.cu:1930-2316
 * ------------------------------------------------------------------------- */
static int pair_oob;

static void pass_vertices(const grid_t *G, const double *d, int *PV, int *PE, int nth) {
    (void)nth;
#pragma omp parallel for schedule(static) num_threads(nth)
    for (int v = 0; v < G->V; v++) {
        int x = v % G->W, y = (v / G->W) % G->H, z = (v / (G->W * G->H)) % G->D;
        double best = DBL_MAX;
        int bid = -1, pid = -1;
        for (int i = 0; i < 14; i++) {
            int nx = x + DIRS[i][0], ny = y + DIRS[i][1], nz = z + DIRS[i][2];
            if (nx < 0 || nx >= G->W || ny < 0 || ny >= G->H || nz < 0 || nz >= G->D) continue;
            int n = nx + ny * G->W + nz * G->W * G->H;
            int e = edge_id(G, x, y, z, nx, ny, nz);
            if ((d[n] < d[v] || (d[n] == d[v] && n < v)) && (d[n] < best || (d[n] == best && n < bid))) {
                best = d[n];
                bid = n;
                pid = e;
            }
        }
        if (pid != -1) {
            PV[v] = pid;
            PE[pid] = v;
        }
    }
}

static void pass_edges(const grid_t *G, const double *d, int *PE, int *PF, int a2, int nth) {
    (void)nth;
#pragma omp parallel for schedule(static) num_threads(nth)
    for (int e = 0; e < G->E; e++) {
        if (PE[e] != -1) continue;
        int v1, v2;
        edge_verts(G, e, &v1, &v2);
        int x1, y1, z1, x2, y2, z2;
        coords(G, v1, &x1, &y1, &z1);
        coords(G, v2, &x2, &y2, &z2);
        double best = DBL_MAX;
        int bid = INT_MAX, pid = -1;
        for (int i = 0; i < 14; i++) {
            int nx = x1 + DIRS[i][0], ny = y1 + DIRS[i][1], nz = z1 + DIRS[i][2];
            int n = nx + ny * G->W + nz * (G->H * G->W);
            if (!is_dir(nx - x2, ny - y2, nz - z2)) continue;
            if (!(nx >= 0 && nx < G->W && ny >= 0 && ny < G->H && nz >= 0 && nz < G->D && n < G->V && n >= 0)) continue;
            int tri = tri_id(G, v1, v2, n);
            if (a2 == 0) {
                if (d[n] > d[v1] || (d[n] == d[v1] && n > v1)) continue;
                if (d[n] > d[v2] || (d[n] == d[v2] && n > v2)) continue;
                if (d[n] < best || (d[n] == best && n < bid)) {
                    best = d[n];
                    bid = n;
                    pid = tri;
                }
            } else {
                int c1 = d[v1] > d[n] || (d[v1] == d[n] && v1 > n);
                int c2 = d[v2] > d[n] || (d[v2] == d[n] && v2 > n);
                if (c1 != c2 && (d[n] < best || (d[n] == best && n < bid))) {
                    best = d[n];
                    bid = n;
                    pid = tri;
                }
            }
        }
        if (pid != -1) {
            if (pid < 0 || pid >= G->F) {
#pragma omp atomic
                pair_oob++;
                continue;
            }
            if (PF[pid] == -1) {
                PE[e] = pid;
                PF[pid] = e;
            }
        }
    }
}

static void pass_faces(const grid_t *G, const double *d, int *PF, int *PT, int a2, int nth) {
    (void)nth;
#pragma omp parallel for schedule(static) num_threads(nth)
    for (int t = 0; t < G->F; t++) {
        if (PF[t] != -1) continue;
        int v1, v2, v3;
        tri_verts(G, t, &v1, &v2, &v3);
        int x1, y1, z1, x2, y2, z2, x3, y3, z3;
        coords(G, v1, &x1, &y1, &z1);
        coords(G, v2, &x2, &y2, &z2);
        coords(G, v3, &x3, &y3, &z3);
        double best = DBL_MAX;
        int bid = INT_MAX, pid = -1;
        for (int i = 0; i < 14; i++) {
            int nx = x1 + DIRS[i][0], ny = y1 + DIRS[i][1], nz = z1 + DIRS[i][2];
            int n = nx + ny * G->W + nz * G->W * G->H;
            if (nx >= G->W || ny >= G->H || nz >= G->D || nx < 0 || ny < 0 || nz < 0 || n >= G->V || n < 0) continue;
            if (!is_dir(nx - x2, ny - y2, nz - z2) || !is_dir(nx - x3, ny - y3, nz - z3)) continue;
            if (n == v1 || n == v2 || n == v3) continue;
            int tet = tet_id(G, v1, v2, v3, n);
            if (a2 == 0) {
                if (d[n] > d[v1] || (d[n] == d[v1] && n > v1)) continue;
                if (d[n] > d[v2] || (d[n] == d[v2] && n > v2)) continue;
                if (d[n] > d[v3] || (d[n] == d[v3] && n > v3)) continue;
                if (d[n] < best || (d[n] == best && n < bid)) {
                    best = d[n];
                    bid = n;
                    pid = tet;
                }
            } else {
                int c1 = d[v1] > d[n] || (d[v1] == d[n] && v1 > n);
                int c2 = d[v2] > d[n] || (d[v2] == d[n] && v2 > n);
                int c3 = d[v3] > d[n] || (d[v3] == d[n] && v3 > n);
                if (((c1 && c2 && !c3) || (c1 && !c2 && c3) || (!c1 && c2 && c3)) &&
                    (d[n] < best || (d[n] == best && n < bid))) {
                    best = d[n];
                    bid = n;
                    pid = tet;
                }
            }
        }
        if (pid != -1) {
            if (pid < 0 || pid >= G->T) {
#pragma omp atomic
                pair_oob++;
                continue;
            }
            if (PT[pid] == -1) {
                PF[t] = pid;
                PT[pid] = t;
            }
        }
    }
}

static int pair_all(const grid_t *G, const double *d, int *PV, int *PE, int *PF, int *PT, int nth) {
    if (nth < 1) nth = 1;
    memset(PV, 0xff, sizeof(int) * (size_t)G->V);
    memset(PE, 0xff, sizeof(int) * (size_t)G->E);
    memset(PF, 0xff, sizeof(int) * (size_t)G->F);
    memset(PT, 0xff, sizeof(int) * (size_t)G->T);
    pair_oob = 0;
    pass_vertices(G, d, PV, PE, nth);
    pass_edges(G, d, PE, PF, 0, nth);
    pass_faces(G, d, PF, PT, 0, nth);
    pass_edges(G, d, PE, PF, 1, nth);
    pass_faces(G, d, PF, PT, 1, nth);
    return pair_oob;
}

int orc_pair(int W, int H, int D, const double *data, int *PV, int *PE, int *PF, int *PT, int nthreads) {
    grid_t G;
    grid_init(&G, W, H, D);
    return pair_all(&G, data, PV, PE, PF, PT, nthreads);
}

/* ---------------------------------------------------------------------------
 * A6: critical-cell mismatch (get_false_*), main_3d.cu:2492-2550
 * ------------------------------------------------------------------------- */
static int xor_crit(int p, int q) { return (q == -1 && p != -1) || (q != -1 && p == -1); }

/* vertex at the componentwise minimum of n vertices */
static int anchor_of(const grid_t *G, const int *vs, int n) {
    int mx = 1 << 30, my = 1 << 30, mz = 1 << 30;
    for (int i = 0; i < n; i++) {
        int x, y, z;
        x = vs[i] % G->W;
        y = (vs[i] / G->W) % G->H;
        z = vs[i] / (G->W * G->H);
        if (x < mx) mx = x;
        if (y < my) my = y;
        if (z < mz) mz = z;
    }
    return mx + my * G->W + mz * G->W * G->H;
}

void orc_cp_mismatch(int W, int H, int D, const int *PV, const int *PE, const int *PF, const int *PT,
                     const int *QV, const int *QE, const int *QF, const int *QT, int counts[4], int *lmin,
                     int *lsad, int *l2sad, int *lmax) {
    grid_t G;
    grid_init(&G, W, H, D);
    int n = 0;
    for (int i = 0; i < G.V; i++)
        if (xor_crit(PV[i], QV[i])) {
            if (lmin) lmin[n] = i;
            n++;
        }
    counts[0] = n;
    n = 0;
    for (int i = 0; i < G.E; i++)
        if (xor_crit(PE[i], QE[i])) {
            if (lsad) lsad[n] = i;
            n++;
        }
    counts[1] = n;
    n = 0;
    for (int i = 0; i < G.F; i++)
        if (xor_crit(PF[i], QF[i])) {
            if (l2sad) l2sad[n] = i;
            n++;
        }
    counts[2] = n;
    n = 0;
    for (int i = 0; i < G.T; i++)
        if (xor_crit(PT[i], QT[i])) {
            if (lmax) lmax[n] = i;
            n++;
        }
    counts[3] = n;
}

/* ---------------------------------------------------------------------------
 * A8: fix_minimum, main_3d.cu:2554-2586
 * ------------------------------------------------------------------------- */
static void fix_minimum(ctx_t *c, int id) {
    if (PVa(id) != -1) {
        int edge = PVa(id);
        int vertex, v2;
        edge_verts(&c->G, edge, &vertex, &v2);
        if (vertex != id) v2 = vertex;
        lower(c, v2);
    } else {
        lower(c, id);
    }
}

/* ---------------------------------------------------------------------------
 * A9: fix_saddle, main_3d.cu:2588-3037
 * ------------------------------------------------------------------------- */
static void fix_saddle(ctx_t *c, int id) {
    const grid_t *G = &c->G;
    int edge = id;
    if (PEa(id) != -1) {
        /* false positive: regular originally, critical in the decompressed field */
        int pe = PEa(id);
        if (pe < G->V && pe >= 0 && pe != -1 && PVa(pe) == id) {
            int v1, v2;
            edge_verts(G, edge, &v1, &v2);
            if (v2 != pe) v1 = pe;
            else {
                v2 = v1;
                v1 = pe;
            }
            int q = QVa(v1);
            if (q == -1 || q < 0 || q >= G->E) return;
            int false_edge = q;
            int fv1, fv2;
            edge_verts(G, false_edge, &fv1, &fv2);
            int false_v2 = v1 == fv1 ? fv2 : fv1;
            double a = gv(c, v2), b = gv(c, false_v2);
            if (a > b || (a == b && v2 > false_v2)) lower(c, v2);
        } else if (pe != -1 && pe < G->F && pe >= 0 && PFa(pe) == id) {
            int face = pe;
            int v1, v2;
            edge_verts(G, edge, &v1, &v2);
            int a, b, v3;
            tri_verts(G, face, &a, &b, &v3);
            v3 = third_of(a, b, v3, v1, v2);
            int other_sortedV1 = !above_g(c, v1, v3) ? v3 : v1;
            int other_sortedV1_1 = !above_g(c, v2, v3) ? v3 : v2;
            int v1_edge = above_g(c, v1, v3);
            int v2_edge = above_g(c, v2, v3);
            int o_v1_edge = above_f(c, v1, v3);
            int o_v2_edge = above_f(c, v2, v3);
            if (v1_edge && v2_edge) {
                lower(c, v3);
            } else if (o_v1_edge && o_v2_edge) {
                lower(c, v3);
            } else {
                int pe2 = PEa(id);
                if (pe2 != -1 && pe2 < G->F && pe2 >= 0 && QFa(pe2) != -1 && QEa(QFa(pe2)) == pe2) {
                    int false_edge = QFa(pe2);
                    edge = false_edge;
                    int a1, b1;
                    edge_verts(G, false_edge, &a1, &b1);
                    int false_v = (a1 != v1 && a1 != v2) ? a1 : b1;
                    double diff = get_delta(c, false_v);
                    /* inner scope: endpoints of the false edge shadow v1, v2 */
                    int w1, w2;
                    edge_verts(G, edge, &w1, &w2);
                    int p, q, w3;
                    tri_verts(G, face, &p, &q, &w3);
                    w3 = third_of(p, q, w3, w1, w2);
                    o_v1_edge = above_f(c, w2, w3);
                    o_v2_edge = above_f(c, w1, w3);
                    if (o_v1_edge && o_v2_edge && PEa(false_edge) != -1 && PFa(PEa(false_edge)) == false_edge) {
                        int f_id = PEa(false_edge);
                        int r, s, u3;
                        tri_verts(G, f_id, &r, &s, &u3);
                        u3 = third_of(r, s, u3, w1, w2);
                        lower(c, u3);
                    } else if (fabs(diff) > 0) {
                        lower(c, false_v);
                    }
                } else {
                    if (o_v1_edge && !v1_edge) lower(c, other_sortedV1);
                    else lower(c, other_sortedV1_1);
                }
            }
        }
    } else {
        /* false negative: critical originally, regular in the decompressed field */
        int qe = QEa(id);
        if (qe != -1 && qe < G->V && qe >= 0 && QVa(qe) == id) {
            lower(c, qe);
        } else if (qe != -1 && qe < G->F && qe >= 0 && QFa(qe) == id) {
            int face = qe;
            int v1, v2;
            edge_verts(G, edge, &v1, &v2);
            int a, b, v3;
            tri_verts(G, face, &a, &b, &v3);
            v3 = third_of(a, b, v3, v1, v2);
            int v1_edge = above_g(c, v2, v3);
            int v2_edge = above_g(c, v1, v3);
            int or_v1_edge = above_f(c, v2, v3);
            int or_v2_edge = above_f(c, v1, v3);
            if (v1_edge == v2_edge) {
                if (v1_edge != or_v1_edge) lower(c, v2);
                if (v2_edge != or_v2_edge) lower(c, v1);
            } else {
                if (PEa(id) != -1) {
                    /* unreachable in this branch (PE[id] == -1), kept literal */
                    int t = PEa(id);
                    if (t >= 0 && t < G->V && PVa(t) == id) {
                        int m = v1;
                        if (v1 == t) m = v2;
                        lower(c, m);
                    }
                } else {
                    /* 14x14 rescan of the edge's cofaces on the ORIGINAL field */
                    int x1, y1, z1, x2, y2, z2;
                    coords(G, v1, &x1, &y1, &z1);
                    coords(G, v2, &x2, &y2, &z2);
                    double best = DBL_MAX;
                    int gid = INT_MAX, pid = -1;
                    for (int i = 0; i < 14; i++) {
                        int nx = x1 + DIRS[i][0], ny = y1 + DIRS[i][1], nz = z1 + DIRS[i][2];
                        int n = nx + ny * G->W + nz * (G->H * G->W);
                        if (!is_dir(nx - x2, ny - y2, nz - z2)) continue;
                        if (!(nx >= 0 && nx < G->W && ny >= 0 && ny < G->H && nz >= 0 && nz < G->D && n < G->V && n >= 0))
                            continue;
                        int tri = tri_id(G, v1, v2, n);
                        int c1 = above_f(c, v1, n), c2 = above_f(c, v2, n);
                        if (c1 != c2) {
                            double fn = fv(c, n);
                            if (fn < best || (fn == best && n < gid)) {
                                best = fn;
                                gid = n;
                                pid = tri;
                            }
                        }
                    }
                    if (pid != -1) {
                        lower(c, gid);
                    } else {
                        lower(c, v1);
                        lower(c, v2);
                    }
                }
            }
        }
    }
}

/* ---------------------------------------------------------------------------
 * A10: fix_2saddle, main_3d.cu:3039-3983
 * ------------------------------------------------------------------------- */
static void fix_2saddle(ctx_t *c, int id) {
    const grid_t *G = &c->G;
    int face = id;
    if (PFa(id) != -1) {
        int pf = PFa(id);
        if (pf < G->E && pf >= 0 && PEa(pf) == id) {
            /* originally paired with an edge */
            int edge = pf;
            int v1, v2;
            edge_verts(G, edge, &v1, &v2);
            int a, b, v3;
            tri_verts(G, face, &a, &b, &v3);
            v3 = third_of(a, b, v3, v1, v2);
            int v1_edge = above_g(c, v2, v3);
            int v2_edge = above_g(c, v1, v3);
            int o_v1_edge = above_f(c, v2, v3);
            int o_v2_edge = above_f(c, v1, v3);
            if (v1_edge && v2_edge) {
                int f_id = PEa(edge);
                if (f_id == -1 || PFa(f_id) != edge) return;
                face = f_id;
                int p, q, w3;
                tri_verts(G, face, &p, &q, &w3);
                w3 = third_of(p, q, w3, v1, v2);
                lower(c, w3);
            } else if (o_v1_edge != o_v2_edge && v1_edge != v2_edge) {
                int f_id = QEa(edge);
                if (f_id == -1 || (f_id != -1 && QFa(QEa(edge)) != edge)) {
                    lower(c, v3);
                } else if (QEa(edge) < G->F && QEa(edge) >= 0) {
                    int p, q, v3_1;
                    tri_verts(G, f_id, &p, &q, &v3_1);
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
        } else if (pf != -1 && pf < G->T && pf >= 0 && PTa(pf) == id) {
            /* originally paired with a tetrahedron */
            int tet = pf;
            int v1, v2, v3;
            tri_verts(G, id, &v1, &v2, &v3);
            int a, b, cc, v4;
            tet_verts(G, tet, &a, &b, &cc, &v4);
            v4 = fourth_of(a, b, cc, v4, v1, v2, v3);
            int or_f1 = above_f(c, v3, v4);
            int or_f2 = above_f(c, v2, v4);
            int or_f3 = above_f(c, v1, v4);
            if (!or_f1 || !or_f2 || !or_f3) {
                int pff = QTa(tet);
                if (pff != -1) {
                    int v1_1, v2_1, v3_1;
                    tri_verts(G, pff, &v1_1, &v2_1, &v3_1);
                    int f1 = above_g(c, v3_1, v4), f2 = above_g(c, v2_1, v4), f3 = above_g(c, v1_1, v4);
                    int o1 = above_f(c, v3_1, v4), o2 = above_f(c, v2_1, v4), o3 = above_f(c, v1_1, v4);
                    if ((!f1 || !f2 || !f3) && (!o1 || !o2 || !o3)) {
                        int id2 = PFa(pff);
                        if (id2 >= 0 && id2 < G->E && PEa(id2) == pff) {
                            int w1, w2;
                            edge_verts(G, id2, &w1, &w2);
                            int w3 = v3_1;
                            if (v1_1 != w1 && w2 != v1_1) w3 = v1_1;
                            else if (v2_1 != w1 && v2_1 != w2) w3 = v2_1;
                            lower(c, w3);
                        } else if (id2 >= 0 && id2 < G->T && PTa(id2) == pff) {
                            int t1, t2, t3, t4;
                            tet_verts(G, id2, &t1, &t2, &t3, &t4);
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
        int qf = QFa(id);
        if (qf != -1 && qf < G->E && QEa(qf) == id) {
            /* decompressed: paired with an edge */
            int edge_id = qf;
            int v1, v2;
            edge_verts(G, edge_id, &v1, &v2);
            int sV1 = !above_g(c, v1, v2) ? v2 : v1;
            int sV2 = !above_g(c, v1, v2) ? v1 : v2;
            int true_face_id = PEa(edge_id);
            if (true_face_id != -1 && PFa(true_face_id) == edge_id) {
                int p, q, w3;
                tri_verts(G, true_face_id, &p, &q, &w3);
                if (sV1 != p && sV2 != p) w3 = p;
                if (sV1 != q && sV2 != q) w3 = q;
                lower(c, w3);
            } else if (true_face_id >= 0 && true_face_id < G->V && PVa(true_face_id) == edge_id) {
                lower(c, sV1);
                lower(c, sV2);
            }
        } else if (qf != -1 && qf < G->T && QTa(qf) == id) {
            /* decompressed: paired with a tetrahedron */
            int tet = qf;
            int v1, v2, v3;
            tri_verts(G, face, &v1, &v2, &v3);
            int a, b, cc, v4;
            tet_verts(G, tet, &a, &b, &cc, &v4);
            v4 = fourth_of(a, b, cc, v4, v1, v2, v3);
            int f1 = above_g(c, v3, v4), f2 = above_g(c, v2, v4), f3 = above_g(c, v1, v4);
            int o1 = above_f(c, v3, v4), o2 = above_f(c, v2, v4), o3 = above_f(c, v1, v4);
            if (f1 && f2 && f3) {
                if (f1 != o1) lower(c, v3);
                else if (f2 != o2) lower(c, v2);
                else if (f3 != o3) lower(c, v1);
            } else {
                int true_cell = PTa(tet);
                if (true_cell >= 0 && true_cell < G->T) {
                    lower(c, v1);
                    lower(c, v2);
                    lower(c, v3);
                } else {
                    int m = smallest_vertex(c, v1, v2, v3);
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

/* ---------------------------------------------------------------------------
 * A11: fix_maximum, main_3d.cu:3985-4303
 * ------------------------------------------------------------------------- */
static void fix_maximum(ctx_t *c, int id) {
    const grid_t *G = &c->G;
    if (PTa(id) != -1) {
        int face1 = PTa(id);
        int v1, v2, v3;
        tri_verts(G, face1, &v1, &v2, &v3);
        int a, b, cc, v4;
        tet_verts(G, id, &a, &b, &cc, &v4);
        v4 = fourth_of(a, b, cc, v4, v1, v2, v3);
        int o1 = above_f(c, v1, v4), o2 = above_f(c, v2, v4), o3 = above_f(c, v3, v4);
        if (o1 && o2 && o3) {
            lower_guarded(c, v4);
        } else {
            int false_cell = QFa(face1);
            if (false_cell >= 0) {
                if (false_cell < G->E && QEa(false_cell) == face1) {
                    int e1, e2;
                    edge_verts(G, false_cell, &e1, &e2);
                    int s1 = above_g(c, e1, e2) ? e1 : e2;
                    lower(c, s1);
                } else if (false_cell < G->T && QTa(false_cell) == face1) {
                    lower_guarded(c, v4);
                }
            }
        }
    } else {
        int face1 = QTa(id);
        int v1, v2, v3;
        tri_verts(G, face1, &v1, &v2, &v3);
        int a, b, cc, v4;
        tet_verts(G, id, &a, &b, &cc, &v4);
        v4 = fourth_of(a, b, cc, v4, v1, v2, v3);
        int f1 = above_g(c, v1, v4), f2 = above_g(c, v2, v4), f3 = above_g(c, v3, v4);
        int o1 = above_f(c, v1, v4), o2 = above_f(c, v2, v4), o3 = above_f(c, v3, v4);
        if (f1 && f2 && f3) {
            if (!o1 && f1) lower(c, v1);
            if (!o2 && f2) lower(c, v2);
            if (!o3 && f3) lower(c, v3);
            if (o1 && o2 && o3) {
                int it = PFa(face1);
                if (it != -1) {
                    int p, q, r, w4;
                    if (it < 0 || it >= G->T) c->oob++; /* a non-tet id read as a tet (reference quirk) */
                    tet_verts(G, it, &p, &q, &r, &w4);
                    w4 = fourth_of(p, q, r, w4, v1, v2, v3);
                    lower(c, w4);
                }
            }
        } else {
            if (PFa(face1) != -1) {
                int pid = PFa(face1);
                if (pid >= 0 && pid < G->E && PEa(pid) == face1) {
                    int e1, e2;
                    edge_verts(G, pid, &e1, &e2);
                    lower(c, e1);
                    lower(c, e2);
                } else {
                    int p, q, r, s;
                    if (pid < 0 || pid >= G->T) c->oob++;
                    tet_verts(G, pid, &p, &q, &r, &s);
                    lower(c, p);
                    lower(c, q);
                    lower(c, r);
                    lower(c, s);
                }
            } else {
                if (!o1) lower(c, v1);
                if (!o2) lower(c, v2);
                if (!o3) lower(c, v3);
            }
        }
    }
}

int orc_fix_cp(int W, int H, int D, const double *f, const double *g, const int *cnt, double bound, double range,
               int edit_type, int preserve_saddles, const int *PV, const int *PE, const int *PF, const int *PT,
               const int *QV, const int *QE, const int *QF, const int *QT, const int counts[4], const int *lmin,
               const int *lsad, const int *l2sad, const int *lmax, double *buf) {
    ctx_t c;
    memset(&c, 0, sizeof(c));
    grid_init(&c.G, W, H, D);
    c.f = f; c.g = g; c.cnt = cnt;
    c.PV = PV; c.PE = PE; c.PF = PF; c.PT = PT;
    c.QV = QV; c.QE = QE; c.QF = QF; c.QT = QT;
    c.bound = bound; c.range = range; c.sentinel = -2000.0 * range;
    c.edit_type = edit_type;
    c.buf = buf;
    /* main_3d.cu:6805-6831: min, [saddle, 2-saddle], max */
    for (int i = 0; i < counts[0]; i++) fix_minimum(&c, lmin[i]);
    if (preserve_saddles == 1) {
        for (int i = 0; i < counts[1]; i++) fix_saddle(&c, lsad[i]);
        for (int i = 0; i < counts[2]; i++) fix_2saddle(&c, l2sad[i]);
    }
    for (int i = 0; i < counts[3]; i++) fix_maximum(&c, lmax[i]);
    return c.oob;
}

/* ---------------------------------------------------------------------------
 * A12/A13: geometry-mode separatrix detection
 * ------------------------------------------------------------------------- */

/* get_cell_tetra, main_3d.cu:4363-4430: cofaces of a face in search order;
 * x = first found, y = last found (left untouched when there is only one) */
static void cell_tetra(ctx_t *c, int face, int *x, int *y) {
    const grid_t *G = &c->G;
    int v1, v2, v3;
    tri_verts(G, face, &v1, &v2, &v3);
    int x1, y1, z1, x2, y2, z2, x3, y3, z3;
    coords(G, v1, &x1, &y1, &z1);
    coords(G, v2, &x2, &y2, &z2);
    coords(G, v3, &x3, &y3, &z3);
    int num = 0;
    for (int i = 0; i < 14; i++) {
        int nx = x1 + DIRS[i][0], ny = y1 + DIRS[i][1], nz = z1 + DIRS[i][2];
        int n = nx + ny * G->W + nz * G->W * G->H;
        if (nx >= G->W || ny >= G->H || nz >= G->D || nx < 0 || ny < 0 || nz < 0 || n >= G->V || n < 0) continue;
        if (!is_dir(nx - x2, ny - y2, nz - z2) || !is_dir(nx - x3, ny - y3, nz - z3)) continue;
        if (n == v1 || n == v2 || n == v3) continue;
        int tid = tet_id(G, v1, v2, v3, n);
        if (num == 0) {
            *x = tid;
            num++;
        } else {
            *y = tid;
        }
    }
}

#define WALK_CAP 100000000

/* is_false, main_3d.cu:4437-4497; returns 1 and records (id, current) when
 * the original ascending path from tet `id` meets a tet whose pairing differs */
static int is_false(ctx_t *c, int id, int *rec_cur) {
    int cur = id, old, t, dt;
    long long steps = 0;
    do {
        old = cur;
        t = PTa(cur);
        dt = QTa(cur);
        if (t == -1) break;
        if (t != dt) {
            *rec_cur = cur;
            return 1;
        }
        if (PFa(t) == -1 || (PFa(t) != -1 && PTa(PFa(t)) != t)) break;
        int t1 = -1, t2 = -1;
        cell_tetra(c, t, &t1, &t2);
        cur = t1 == cur ? t2 : t1;
        if (++steps > WALK_CAP) {
            c->oob++;
            break;
        }
    } while (cur != old && cur != -1);
    return 0;
}

/* strict descending checks (not the reference's; see orc_set_strict_ds) */
static int g_strict_ds = 0;
void orc_set_strict_ds(int on) { g_strict_ds = on ? 1 : 0; }

/* The whole original descending path from v (steepest-descent pairing PV,
 * the loop of get_false_ds_vpath with dec_current_id advancing as
 * current_id does): the first vertex whose decompressed pairing differs, or
 * -1 when the path reaches a minimum clean. */
static int ds_first_diff(ctx_t *c, int v) {
    const grid_t *G = &c->G;
    for (long long steps = 0;; steps++) {
        const int pv = PVa(v);
        if (pv == -1) return -1;
        if (pv != QVa(v)) return v;
        if (PEa(pv) == -1) return -1;
        int a, b;
        edge_verts(G, pv, &a, &b);
        v = a == v ? b : a;
        if (steps > (long long)G->V) {
            c->oob++;
            return -1;
        }
    }
}

int orc_path_detect(int W, int H, int D, const int *PV, const int *PE, const int *PF, const int *PT,
                    const int *QV, const int *QE, const int *QF, const int *QT, int counts[2], int *as_tet,
                    int *as_cur, int *ds_edge, int *ds_vert) {
    ctx_t cc;
    ctx_t *c = &cc;
    memset(c, 0, sizeof(*c));
    grid_init(&c->G, W, H, D);
    const grid_t *G = &c->G;
    c->PV = PV; c->PE = PE; c->PF = PF; c->PT = PT;
    c->QV = QV; c->QE = QE; c->QF = QF; c->QT = QT;
    /* get_false_as_vpath, main_3d.cu:4540-4610 */
    int nas = 0;
    for (int i = 0; i < G->F; i++) {
        if (PF[i] != -1) continue;
        int v1, v2, v3;
        tri_verts(G, i, &v1, &v2, &v3);
        int x1, y1, z1, x2, y2, z2, x3, y3, z3;
        coords(G, v1, &x1, &y1, &z1);
        coords(G, v2, &x2, &y2, &z2);
        coords(G, v3, &x3, &y3, &z3);
        for (int k = 0; k < 14; k++) {
            int nx = x1 + DIRS[k][0], ny = y1 + DIRS[k][1], nz = z1 + DIRS[k][2];
            int n = nx + ny * G->W + nz * G->W * G->H;
            if (nx >= G->W || ny >= G->H || nz >= G->D || nx < 0 || ny < 0 || nz < 0 || n >= G->V || n < 0) continue;
            if (!is_dir(nx - x2, ny - y2, nz - z2) || !is_dir(nx - x3, ny - y3, nz - z3)) continue;
            if (n == v1 || n == v2 || n == v3) continue;
            int tid = tet_id(G, v1, v2, v3, n);
            int cur;
            if (is_false(c, tid, &cur)) {
                if (as_tet) as_tet[nas] = tid;
                if (as_cur) as_cur[nas] = cur;
                nas++;
                break;
            }
        }
    }
    /* get_false_ds_vpath, main_3d.cu:4837-4959.  dec_current_id never
     * advances, so the walk stops at the second vertex of each path: only the
     * first vertex of each endpoint is compared. */
    int nds = 0;
    for (int i = 0; i < G->E; i++) {
        if (PE[i] != -1) continue;
        int v1, v2;
        edge_verts(G, i, &v1, &v2);
        int ends[2] = {v1, v2};
        for (int k = 0; k < 2; k++) {
            int v = ends[k];
            if (g_strict_ds) {
                const int u = ds_first_diff(c, v);
                if (u >= 0) {
                    if (ds_edge) ds_edge[nds] = i;
                    if (ds_vert) ds_vert[nds] = u;
                    nds++;
                    break;
                }
                continue;
            }
            int pv = PVa(v);
            if (pv == -1) continue;
            if (pv != QVa(v)) {
                if (ds_edge) ds_edge[nds] = i;
                if (ds_vert) ds_vert[nds] = v;
                nds++;
                break;
            }
        }
    }
    counts[0] = nas;
    counts[1] = nds;
    return c->oob;
}

/* ---------------------------------------------------------------------------
 * A18: connectivity-mode separatrices (preserve_vpath=1, preserve_geometry=0)
 * ------------------------------------------------------------------------- */

/* get_paired_id, main_3d.cu:4499-4537: end of the ascending path from tet id
 * under the original (dec = 0) or decompressed (dec = 1) pairing */
static int paired_id(ctx_t *c, int id, int dec) {
    int cur = id, old, t;
    long long steps = 0;
    do {
        old = cur;
        t = dec ? QTa(cur) : PTa(cur);
        if (t == -1) break;
        const int pf = dec ? QFa(t) : PFa(t);
        if (pf == -1 || (pf != -1 && (dec ? QTa(pf) : PTa(pf)) != t)) break;
        int t1 = -1, t2 = -1;
        cell_tetra(c, t, &t1, &t2);
        cur = t1 == cur ? t2 : t1;
        if (++steps > WALK_CAP) {
            c->oob++;
            break;
        }
    } while (cur != old && cur != -1);
    return cur;
}

/* the descending walk of get_orginal_saddle_min_pairs (main_3d.cu:4613-4687)
 * from vertex v0 under the original pairing: the minimum reached */
static int min_of(ctx_t *c, int v0) {
    int v = v0, cur = v0;
    long long steps = 0;
    do {
        v = cur;
        if (PVa(v) == -1) break;
        const int e = PVa(v);
        if (PEa(e) == -1) break;
        int a, b;
        edge_verts(&c->G, e, &a, &b);
        cur = a == cur ? b : a;
        if (++steps > WALK_CAP) {
            c->oob++;
            break;
        }
    } while (PVa(v) != -1);
    return v;
}

/* the decompressed descending walk of get_false_ds_vpath_connectivity
 * (main_3d.cu:4961-5062): end vertex; *trouble (if -1) becomes the first
 * vertex whose original and decompressed pairings differ */
static int dec_min_of(ctx_t *c, int v0, int *trouble) {
    int v = v0, cur = v0;
    long long steps = 0;
    do {
        v = cur;
        if (QVa(v) == -1) break;
        const int e = PVa(v), de = QVa(v);
        if (e != de && *trouble == -1) *trouble = v;
        if (QEa(de) == -1) break;
        int a, b;
        edge_verts(&c->G, de, &a, &b);
        cur = a == cur ? b : a;
        if (++steps > WALK_CAP) {
            c->oob++;
            break;
        }
    } while (QVa(v) != -1);
    return v;
}

/* get_orginal_saddle_min_pairs / get_orginal_saddle_max_pairs
 * (main_3d.cu:4613-4759): the original ends of every original saddle's
 * separatrices; conn_min (2E) by edge, conn_max (2F) by triangle and coface
 * number, -1 where unset.  The reference's max table is indexed by its
 * direction-loop counter instead of the triangle (a race between all
 * triangles); this restates the intended indexing. */
static void conn_prep(ctx_t *c, int *conn_min, int *conn_max) {
    const grid_t *G = &c->G;
    for (int i = 0; i < 2 * G->E; i++) conn_min[i] = -1;
    for (int i = 0; i < 2 * G->F; i++) conn_max[i] = -1;
    for (int i = 0; i < G->E; i++) {
        if (c->PE[i] != -1) continue;
        int v1, v2;
        edge_verts(G, i, &v1, &v2);
        conn_min[2 * i] = min_of(c, v1);
        conn_min[2 * i + 1] = min_of(c, v2);
    }
    for (int i = 0; i < G->F; i++) {
        if (c->PF[i] != -1) continue;
        int v1, v2, v3;
        tri_verts(G, i, &v1, &v2, &v3);
        int x1, y1, z1, x2, y2, z2, x3, y3, z3;
        coords(G, v1, &x1, &y1, &z1);
        coords(G, v2, &x2, &y2, &z2);
        coords(G, v3, &x3, &y3, &z3);
        int num = 0;
        for (int k = 0; k < 14; k++) {
            int nx = x1 + DIRS[k][0], ny = y1 + DIRS[k][1], nz = z1 + DIRS[k][2];
            int n = nx + ny * G->W + nz * G->W * G->H;
            if (nx >= G->W || ny >= G->H || nz >= G->D || nx < 0 || ny < 0 || nz < 0 || n >= G->V || n < 0) continue;
            if (!is_dir(nx - x2, ny - y2, nz - z2) || !is_dir(nx - x3, ny - y3, nz - z3)) continue;
            if (n == v1 || n == v2 || n == v3) continue;
            conn_max[2 * i + num] = paired_id(c, tet_id(G, v1, v2, v3, n), 0);
            num++;
        }
    }
}

/* get_false_as_vpath_connectivity (intended indexing) and
 * get_false_ds_vpath_connectivity, main_3d.cu:4761-4835, 4961-5062 */
static void conn_detect(ctx_t *c, const int *conn_min, const int *conn_max, int counts[2], int *as_tet, int *as_cur,
                        int *ds_edge, int *ds_vert) {
    const grid_t *G = &c->G;
    int nas = 0;
    for (int i = 0; i < G->F; i++) {
        if (c->QF[i] != -1) continue; /* the decompressed 2-saddles */
        int v1, v2, v3;
        tri_verts(G, i, &v1, &v2, &v3);
        int x1, y1, z1, x2, y2, z2, x3, y3, z3;
        coords(G, v1, &x1, &y1, &z1);
        coords(G, v2, &x2, &y2, &z2);
        coords(G, v3, &x3, &y3, &z3);
        int num = 0;
        for (int k = 0; k < 14; k++) {
            int nx = x1 + DIRS[k][0], ny = y1 + DIRS[k][1], nz = z1 + DIRS[k][2];
            int n = nx + ny * G->W + nz * G->W * G->H;
            if (nx >= G->W || ny >= G->H || nz >= G->D || nx < 0 || ny < 0 || nz < 0 || n >= G->V || n < 0) continue;
            if (!is_dir(nx - x2, ny - y2, nz - z2) || !is_dir(nx - x3, ny - y3, nz - z3)) continue;
            if (n == v1 || n == v2 || n == v3) continue;
            const int tid = tet_id(G, v1, v2, v3, n);
            const int dec_id = paired_id(c, tid, 1);
            int cur;
            if (dec_id != conn_max[2 * i + num] && is_false(c, tid, &cur)) {
                if (as_tet) as_tet[nas] = tid;
                if (as_cur) as_cur[nas] = cur;
                nas++;
                break;
            }
            num++;
        }
    }
    int nds = 0;
    for (int i = 0; i < G->E; i++) {
        if (c->PE[i] != -1) continue;
        int v1, v2;
        edge_verts(G, i, &v1, &v2);
        int trouble = -1;
        const int e1 = dec_min_of(c, v1, &trouble);
        int hit = e1 != conn_min[2 * i];
        if (!hit) hit = dec_min_of(c, v2, &trouble) != conn_min[2 * i + 1];
        if (hit) {
            if (ds_edge) ds_edge[nds] = i;
            if (ds_vert) ds_vert[nds] = trouble;
            nds++;
        }
    }
    counts[0] = nas;
    counts[1] = nds;
}

int orc_path_detect_conn(int W, int H, int D, const int *PV, const int *PE, const int *PF, const int *PT,
                         const int *QV, const int *QE, const int *QF, const int *QT, int counts[2], int *as_tet,
                         int *as_cur, int *ds_edge, int *ds_vert) {
    ctx_t cc;
    ctx_t *c = &cc;
    memset(c, 0, sizeof(*c));
    grid_init(&c->G, W, H, D);
    c->PV = PV; c->PE = PE; c->PF = PF; c->PT = PT;
    c->QV = QV; c->QE = QE; c->QF = QF; c->QT = QT;
    int *cmin = (int *)malloc(sizeof(int) * 2 * (size_t)c->G.E);
    int *cmax = (int *)malloc(sizeof(int) * 2 * (size_t)c->G.F);
    conn_prep(c, cmin, cmax);
    conn_detect(c, cmin, cmax, counts, as_tet, as_cur, ds_edge, ds_vert);
    free(cmin);
    free(cmax);
    return c->oob;
}

/* fix_as_vpath (type-2 branch; type 1 is never recorded), main_3d.cu:5135-5244 */
static void fix_as_vpath(ctx_t *c, int t_idx) {
    const grid_t *G = &c->G;
    int true_edge = PTa(t_idx);
    int false_edge = QTa(t_idx);
    int pfe = PFa(false_edge);
    if (pfe >= 0 && pfe < G->T && PTa(pfe) == false_edge) {
        int true_face = pfe;
        int v1, v2, v3;
        tri_verts(G, false_edge, &v1, &v2, &v3);
        int a, b, cc, d;
        tet_verts(G, true_face, &a, &b, &cc, &d);
        int true_v3 = fourth_of(a, b, cc, d, v1, v2, v3);
        lower(c, true_v3);
    } else {
        int v1, v2, v3;
        tri_verts(G, true_edge, &v1, &v2, &v3);
        int a, b, true_v3;
        tri_verts(G, false_edge, &a, &b, &true_v3);
        if (a != v1 && a != v2 && a != v3) true_v3 = a;
        else if (b != v1 && b != v2 && b != v3) true_v3 = b;
        lower(c, true_v3);
    }
}

/* fix_ds_vpath (type-0 branch; type 1 is never recorded), main_3d.cu:5246-5295 */
static void fix_ds_vpath(ctx_t *c, int v_idx) {
    int tpe = PVa(v_idx);
    int v1, v2;
    edge_verts(&c->G, tpe, &v1, &v2);
    int tv = v_idx == v1 ? v2 : v1;
    lower(c, tv);
}

/* ---------------------------------------------------------------------------
 * Walls (preserve_connectors = 1): get_false_ds_wall, main_3d.cu:5064-5121,
 * and fix_ds_wall, main_3d.cu:5297-5413, restated without the races of the
 * reference's detection (all threads of a block share one stack, all threads
 * one spill buffer and one visited array; the record index array aliases the
 * record array; the launch covers only the first V face ids).  Here every
 * original 2-saddle face runs its own depth-first search with its own stack
 * and visited marks, in the reference's order: pop a face; if it was not
 * visited yet, check its edges (v1 v2), (v1 v3), (v2 v3) of its descending
 * vertex triple; an originally critical edge is skipped; the first edge whose
 * original and decompressed pairings differ is the record; otherwise the face
 * the edge is originally paired with (if any, and not this face) is pushed.
 * ------------------------------------------------------------------------- */
static int wall_edges(const grid_t *G, int t, int e[3]) {
    int v1, v2, v3, x1, y1, z1, x2, y2, z2, x3, y3, z3;
    tri_verts(G, t, &v1, &v2, &v3);
    coords(G, v1, &x1, &y1, &z1);
    coords(G, v2, &x2, &y2, &z2);
    coords(G, v3, &x3, &y3, &z3);
    e[0] = edge_id(G, x1, y1, z1, x2, y2, z2);
    e[1] = edge_id(G, x1, y1, z1, x3, y3, z3);
    e[2] = edge_id(G, x2, y2, z2, x3, y3, z3);
    return 3;
}

/* the record edge of 2-saddle `sad`, or -1; stamp[] holds sad + 1 on the
 * faces this search visited */
static int wall_search(ctx_t *c, int sad, int *stamp, int **stack, long long *cap, long long *pops) {
    const grid_t *G = &c->G;
    long long top = 0;
    (*stack)[top++] = sad;
    while (top > 0) {
        const int t = (*stack)[--top];
        (*pops)++;
        if (stamp[t] == sad + 1) continue;
        stamp[t] = sad + 1;
        int e[3];
        wall_edges(G, t, e);
        for (int k = 0; k < 3; k++) {
            const int j = e[k];
            const int pe = PEa(j);
            if (pe == -1) continue;
            if (pe != QEa(j)) return j;
            if (pe != t && pe >= 0 && pe < G->F && PFa(pe) == j) {
                if (top == *cap) {
                    *cap *= 2;
                    *stack = (int *)realloc(*stack, sizeof(int) * (size_t)*cap);
                }
                (*stack)[top++] = pe;
            }
        }
    }
    return -1;
}

static int wall_detect(ctx_t *c, int *w_sad, int *w_edge, long long *pops) {
    const grid_t *G = &c->G;
    int *stamp = (int *)calloc((size_t)G->F, sizeof(int));
    long long cap = 1024;
    int *stack = (int *)malloc(sizeof(int) * (size_t)cap);
    int n = 0;
    for (int i = 0; i < G->F; i++) {
        if (c->PF[i] != -1) continue;
        const int j = wall_search(c, i, stamp, &stack, &cap, pops);
        if (j >= 0) {
            if (w_sad) w_sad[n] = i;
            if (w_edge) w_edge[n] = j;
            n++;
        }
    }
    free(stamp);
    free(stack);
    return n;
}

int orc_wall_detect(int W, int H, int D, const int *PV, const int *PE, const int *PF, const int *PT, const int *QV,
                    const int *QE, const int *QF, const int *QT, int *count, int *w_sad, int *w_edge,
                    long long *pops) {
    ctx_t cc;
    ctx_t *c = &cc;
    memset(c, 0, sizeof(*c));
    grid_init(&c->G, W, H, D);
    c->PV = PV; c->PE = PE; c->PF = PF; c->PT = PT;
    c->QV = QV; c->QE = QE; c->QF = QF; c->QT = QT;
    long long p = 0;
    *count = wall_detect(c, w_sad, w_edge, &p);
    if (pops) *pops = p;
    return c->oob;
}

/* fix_ds_wall, main_3d.cu:5297-5413, for the record edge e */
static void fix_ds_wall(ctx_t *c, int e) {
    const grid_t *G = &c->G;
    const int tf = PEa(e), ff = QEa(e);
    if (tf == ff) return;
    int v1, v2;
    edge_verts(G, e, &v1, &v2);
    if (tf >= 0 && ff >= 0 && tf < G->F && PFa(tf) == e && ff < G->F && QFa(ff) == e) {
        int a, b, v3;
        tri_verts(G, tf, &a, &b, &v3);
        if (a != v1 && a != v2) v3 = a;
        if (b != v1 && b != v2) v3 = b;
        if (fabs(get_delta(c, v3)) > 1e-16 * c->range) {
            lower(c, v3);
        } else {
            lower(c, v1);
            lower(c, v2);
        }
    } else if (tf == -1 || tf >= G->F || (tf >= 0 && PFa(tf) != e)) {
        lower(c, v1);
        lower(c, v2);
    } else if (ff == -1 || ff >= G->F || (ff >= 0 && QFa(ff) != e)) {
        int a, b, v3;
        tri_verts(G, tf, &a, &b, &v3);
        lower(c, third_of(a, b, v3, v1, v2));
    }
}

/* ---------------------------------------------------------------------------
 * A7: applyDeltaBuffer1, main_3d.cu:1122-1164
 * ------------------------------------------------------------------------- */
/* returns 1 when some value or edit counter changed (0: the round was a fixed point) */
static int apply_buffer(const grid_t *G, const double *f, double *g, int *cnt, const double *buf, double bound,
                        double range, int preserve_type) {
    const double sentinel = -2000.0 * range;
    int progress = 0;
    for (int v = 0; v < G->V; v++) {
        if (buf[v] != sentinel) {
            if (preserve_type == 0 && fabs(buf[v]) > 1e-15 * range && cnt[v] < 5 &&
                fabs(f[v] - (g[v] + buf[v])) <= bound) {
                g[v] += buf[v];
                cnt[v] += 1;
                progress = 1;
            } else {
                if (cnt[v] != 6 || g[v] != f[v] - bound) progress = 1;
                cnt[v] = 6;
                g[v] = f[v] - bound;
            }
        }
    }
    return progress;
}

/* Stall breaking (not in the reference, whose loop repeats a round that
 * changed nothing forever): every vertex within `radius` per axis of a seed
 * goes back to its original value.  Seeds are marked 1 in m; the box is grown
 * axis by axis (a vertex joins when a seed of its grid line is within radius). */
static void snap_box(const grid_t *G, const double *f, double *g, unsigned char *m, int radius) {
    const int n3[3] = {G->W, G->H, G->D};
    const long long st3[3] = {1, G->W, (long long)G->W * G->H};
    unsigned char *grow = (unsigned char *)malloc((size_t)G->V);
    for (int ax = 0; ax < 3; ax++) {
        const int n = n3[ax];
        const long long step = st3[ax];
        const int r = radius < n ? radius : n;
        memset(grow, 0, (size_t)G->V);
        for (long long base = 0; base < G->V; base++) {
            /* base runs over the vertices whose coordinate along ax is 0 */
            const int x = (int)(base % G->W), y = (int)((base / G->W) % G->H), z = (int)(base / ((long long)G->W * G->H));
            if ((ax == 0 && x) || (ax == 1 && y) || (ax == 2 && z)) continue;
            for (int i = 0; i < n; i++) {
                if (!m[base + i * step]) continue;
                const int lo = i - r < 0 ? 0 : i - r, hi = i + r > n - 1 ? n - 1 : i + r;
                for (int j = lo; j <= hi; j++) grow[base + j * step] = 1;
            }
        }
        memcpy(m, grow, (size_t)G->V);
    }
    free(grow);
    for (int v = 0; v < G->V; v++)
        if (m[v]) g[v] = f[v];
}

/* the k-th break (k = 0, 1, ...) resets the box of half-width k: the seeds
 * alone first, then growing by one per break, up to the whole grid (where g = f
 * and nothing can mismatch, so every run ends) */
static int stall_radius(const grid_t *G, long long nbreaks) {
    long long span = G->W;
    if (G->H > span) span = G->H;
    if (G->D > span) span = G->D;
    return (int)(nbreaks < span ? nbreaks : span);
}

/* ---------------------------------------------------------------------------
 * A16: the host loop, main_3d.cu:6255-7149
 * ------------------------------------------------------------------------- */
int orc_correct(int W, int H, int D, const double *f, double *g, double rel_eps, const int flags[7], int max_outer,
                int nthreads, long long stats[8], int *cnt_out) {
    long long st9[9];
    const int rc = orc_correct_ex(W, H, D, f, g, rel_eps, flags, max_outer, nthreads, 0, st9, cnt_out);
    memcpy(stats, st9, 8 * sizeof(long long));
    return rc;
}

int orc_correct_ex(int W, int H, int D, const double *f, double *g, double rel_eps, const int flags[7], int max_outer,
                   int nthreads, int break_stalls, long long stats[9], int *cnt_out) {
    return orc_correct_rounds(W, H, D, f, g, rel_eps, flags, max_outer, 0, nthreads, break_stalls, stats, cnt_out);
}

int orc_correct_rounds(int W, int H, int D, const double *f, double *g, double rel_eps, const int flags[7],
                       int max_outer, long long max_rounds, int nthreads, int break_stalls, long long stats[9],
                       int *cnt_out) {
    const int ps = flags[0], pv = flags[1], pg = flags[2], filt = flags[3], pc = flags[4], pt = flags[5],
              et = flags[6];
    for (int i = 0; i < 9; i++) stats[i] = 0;
    long long breaks = 0;
    unsigned char *mark = NULL;
    const int walls = pc == 1 && pv == 1; /* wall checks run in the separatrix phase */
    const int conn = pv == 1 && pg == 0; /* connectivity-mode separatrices */
    if (max_outer <= 0) max_outer = 100000;
    grid_t G;
    grid_init(&G, W, H, D);
    const size_t V = (size_t)G.V;
    double mn = f[0], mx = f[0];
    for (size_t i = 1; i < V; i++) {
        if (f[i] < mn) mn = f[i];
        if (f[i] > mx) mx = f[i];
    }
    const double bound = (mx - mn) * rel_eps; /* main_3d.cu:6307 */
    const double range = mx - mn;             /* main_3d.cu:6309, 6323 */
    const double sentinel = -2000.0 * range;

    int *P = (int *)malloc(sizeof(int) * ((size_t)G.V + G.E + G.F + G.T));
    int *Q = (int *)malloc(sizeof(int) * ((size_t)G.V + G.E + G.F + G.T));
    int *PV = P, *PE = P + G.V, *PF = PE + G.E, *PT = PF + G.F;
    int *QV = Q, *QE = Q + G.V, *QF = QE + G.E, *QT = QF + G.F;
    int *lmin = (int *)malloc(sizeof(int) * (size_t)G.V);
    int *lsad = (int *)malloc(sizeof(int) * (size_t)G.E);
    int *l2s = (int *)malloc(sizeof(int) * (size_t)G.F);
    int *lmax = (int *)malloc(sizeof(int) * (size_t)G.T);
    int *as_tet = (int *)malloc(sizeof(int) * (size_t)G.F);
    int *as_cur = (int *)malloc(sizeof(int) * (size_t)G.F);
    int *ds_e = (int *)malloc(sizeof(int) * (size_t)G.E);
    int *ds_v = (int *)malloc(sizeof(int) * (size_t)G.E);
    int *w_sad = walls ? (int *)malloc(sizeof(int) * (size_t)G.F) : NULL;
    int *w_edge = walls ? (int *)malloc(sizeof(int) * (size_t)G.F) : NULL;
    long long wall_pops = 0;
    int *cnt = (int *)malloc(sizeof(int) * V);
    double *buf = (double *)malloc(sizeof(double) * V);
    long long oob = 0;

    oob += pair_all(&G, f, PV, PE, PF, PT, nthreads);
    for (size_t i = 0; i < V; i++) cnt[i] = 0;
    if (filt == 1) { /* filter_*, main_3d.cu:2405-2490 */
        for (int i = 0; i < G.V; i++)
            if (PV[i] == -1) {
                cnt[i] = 6;
                g[i] = f[i] - bound;
            }
        for (int i = 0; i < G.E; i++)
            if (PE[i] == -1) {
                int a, b;
                edge_verts(&G, i, &a, &b);
                g[a] = f[a] - bound; g[b] = f[b] - bound;
                cnt[a] = cnt[b] = 6;
            }
        for (int i = 0; i < G.F; i++)
            if (PF[i] == -1) {
                int a, b, cc;
                tri_verts(&G, i, &a, &b, &cc);
                g[a] = f[a] - bound; g[b] = f[b] - bound; g[cc] = f[cc] - bound;
                cnt[a] = cnt[b] = cnt[cc] = 6;
            }
        for (int i = 0; i < G.T; i++)
            if (PT[i] == -1) {
                int a, b, cc, d;
                tet_verts(&G, i, &a, &b, &cc, &d);
                g[a] = f[a] - bound; g[b] = f[b] - bound; g[cc] = f[cc] - bound; g[d] = f[d] - bound;
                cnt[a] = cnt[b] = cnt[cc] = cnt[d] = 6;
            }
    }
    oob += pair_all(&G, g, QV, QE, QF, QT, nthreads);
    int cc4[4];
    orc_cp_mismatch(W, H, D, PV, PE, PF, PT, QV, QE, QF, QT, cc4, lmin, lsad, l2s, lmax);
    stats[4] = cc4[0]; stats[5] = cc4[1]; stats[6] = cc4[2]; stats[7] = cc4[3];
    for (size_t i = 0; i < V; i++) cnt[i] = 1; /* init_counter runs after the filters */

    int *cmin = NULL, *cmax = NULL;
    int n_as = 1, n_ds = 1, n_wall = 1;
    long long total_ite = 0, cp_ite = 0, rounds = 0;
    const long long round_cap = max_rounds > 0 ? max_rounds : (long long)max_outer * 64;
    int converged = 1;
    ctx_t c;
    memset(&c, 0, sizeof(c));
    c.G = G;
    c.f = f; c.g = g; c.cnt = cnt;
    c.PV = PV; c.PE = PE; c.PF = PF; c.PT = PT;
    c.QV = QV; c.QE = QE; c.QF = QF; c.QT = QT;
    c.bound = bound; c.range = range; c.sentinel = sentinel; c.edit_type = et; c.buf = buf;
    if (conn) { /* main_3d.cu:6566-6582, after the original pairing */
        cmin = (int *)malloc(sizeof(int) * 2 * (size_t)G.E);
        cmax = (int *)malloc(sizeof(int) * 2 * (size_t)G.F);
        conn_prep(&c, cmin, cmax);
        oob += c.oob;
    }

    while (n_as > 0 || n_ds > 0 || n_wall > 0 || cc4[2] > 0 || cc4[3] > 0 || cc4[0] > 0 || cc4[1] > 0) {
        if (total_ite >= max_outer || rounds >= round_cap) {
            converged = 0;
            break;
        }
        total_ite++;
        while (cc4[3] > 0 || cc4[2] > 0 || cc4[0] > 0 || cc4[1] > 0) {
            if (rounds >= round_cap) break;
            rounds++;
            cp_ite++;
            for (size_t i = 0; i < V; i++) buf[i] = sentinel;
            c.oob = 0;
            for (int i = 0; i < cc4[0]; i++) fix_minimum(&c, lmin[i]);
            if (cc4[1] > 0 && ps == 1)
                for (int i = 0; i < cc4[1]; i++) fix_saddle(&c, lsad[i]);
            if (cc4[2] > 0 && ps == 1)
                for (int i = 0; i < cc4[2]; i++) fix_2saddle(&c, l2s[i]);
            for (int i = 0; i < cc4[3]; i++) fix_maximum(&c, lmax[i]);
            oob += c.oob;
            const int progress = apply_buffer(&G, f, g, cnt, buf, bound, range, pt);
            oob += pair_all(&G, g, QV, QE, QF, QT, nthreads);
            orc_cp_mismatch(W, H, D, PV, PE, PF, PT, QV, QE, QF, QT, cc4, lmin, lsad, l2s, lmax);
            if (ps != 1) cc4[1] = cc4[2] = 0;
            if (break_stalls && !progress && rounds < round_cap &&
                (cc4[0] > 0 || cc4[1] > 0 || cc4[2] > 0 || cc4[3] > 0)) {
                /* seeds: the vertices of the remaining mismatched cells */
                if (!mark) mark = (unsigned char *)malloc(V);
                memset(mark, 0, V);
                for (int i = 0; i < cc4[0]; i++) mark[lmin[i]] = 1;
                for (int i = 0; i < cc4[1]; i++) {
                    int a, b;
                    edge_verts(&G, lsad[i], &a, &b);
                    mark[a] = mark[b] = 1;
                }
                for (int i = 0; i < cc4[2]; i++) {
                    int a, b, c3;
                    tri_verts(&G, l2s[i], &a, &b, &c3);
                    mark[a] = mark[b] = mark[c3] = 1;
                }
                for (int i = 0; i < cc4[3]; i++) {
                    int a, b, c3, d;
                    tet_verts(&G, lmax[i], &a, &b, &c3, &d);
                    mark[a] = mark[b] = mark[c3] = mark[d] = 1;
                }
                snap_box(&G, f, g, mark, stall_radius(&G, breaks));
                breaks++;
                oob += pair_all(&G, g, QV, QE, QF, QT, nthreads);
                orc_cp_mismatch(W, H, D, PV, PE, PF, PT, QV, QE, QF, QT, cc4, lmin, lsad, l2s, lmax);
                if (ps != 1) cc4[1] = cc4[2] = 0;
            }
        }
        if (rounds >= round_cap) {
            converged = 0;
            break;
        }
        if (pv == 0) break;
        /* separatrix phase, main_3d.cu:6943-7148 */
        int pc2[2] = {0, 0};
        if (conn) {
            c.oob = 0;
            conn_detect(&c, cmin, cmax, pc2, as_tet, as_cur, ds_e, ds_v);
            oob += c.oob;
        } else {
            oob += orc_path_detect(W, H, D, PV, PE, PF, PT, QV, QE, QF, QT, pc2, as_tet, as_cur, ds_e, ds_v);
        }
        n_as = pc2[0];
        n_ds = pc2[1];
        n_wall = walls ? wall_detect(&c, w_sad, w_edge, &wall_pops) : 0;
        rounds++;
        for (size_t i = 0; i < V; i++) buf[i] = sentinel;
        c.oob = 0;
        for (int i = 0; i < n_as; i++) fix_as_vpath(&c, as_cur[i]);
        for (int i = 0; i < n_ds; i++) fix_ds_vpath(&c, ds_v[i]);
        for (int i = 0; i < n_wall; i++) fix_ds_wall(&c, w_edge[i]);
        oob += c.oob;
        const int progress = apply_buffer(&G, f, g, cnt, buf, bound, range, pt);
        oob += pair_all(&G, g, QV, QE, QF, QT, nthreads);
        orc_cp_mismatch(W, H, D, PV, PE, PF, PT, QV, QE, QF, QT, cc4, lmin, lsad, l2s, lmax);
        if (break_stalls && !progress && rounds < round_cap && n_as + n_ds + n_wall > 0) {
            /* seeds: the records' current tetrahedra and trouble makers */
            if (!mark) mark = (unsigned char *)malloc(V);
            memset(mark, 0, V);
            for (int i = 0; i < n_as; i++) {
                int a, b, c3, d;
                tet_verts(&G, as_cur[i], &a, &b, &c3, &d);
                mark[a] = mark[b] = mark[c3] = mark[d] = 1;
            }
            for (int i = 0; i < n_ds; i++)
                if (ds_v[i] >= 0 && ds_v[i] < G.V) mark[ds_v[i]] = 1;
            for (int i = 0; i < n_wall; i++) {
                int a, b;
                edge_verts(&G, w_edge[i], &a, &b);
                mark[a] = mark[b] = 1;
            }
            snap_box(&G, f, g, mark, stall_radius(&G, breaks));
            breaks++;
            oob += pair_all(&G, g, QV, QE, QF, QT, nthreads);
            orc_cp_mismatch(W, H, D, PV, PE, PF, PT, QV, QE, QF, QT, cc4, lmin, lsad, l2s, lmax);
        }
        n_as = n_ds = n_wall = 0;
        if (cc4[0] == 0 && cc4[1] == 0 && cc4[2] == 0 && cc4[3] == 0) {
            if (conn) {
                c.oob = 0;
                conn_detect(&c, cmin, cmax, pc2, as_tet, as_cur, ds_e, ds_v);
                oob += c.oob;
            } else {
                oob += orc_path_detect(W, H, D, PV, PE, PF, PT, QV, QE, QF, QT, pc2, as_tet, as_cur, ds_e, ds_v);
            }
            n_as = pc2[0];
            n_ds = pc2[1];
            n_wall = walls ? wall_detect(&c, w_sad, w_edge, &wall_pops) : 0;
        }
    }
    stats[0] = total_ite;
    stats[1] = cp_ite;
    stats[2] = oob;
    stats[3] = converged;
    stats[8] = breaks;
    if (cnt_out) memcpy(cnt_out, cnt, sizeof(int) * V);
    free(mark);
    free(P); free(Q); free(lmin); free(lsad); free(l2s); free(lmax);
    free(as_tet); free(as_cur); free(ds_e); free(ds_v); free(cnt); free(buf);
    free(w_sad); free(w_edge);
    free(cmin); free(cmax);
    return 0;
}

/* ---------------------------------------------------------------------------
 * N4: manifold labels of one field, by following the reference's path rules
 * serially (descending: processVertices pairing; ascending: is_false's walk,
 * main_3d.cu:4437-4497).  desc[v] = minimum reached, asc[t] = maximum reached
 * or -1 when the walk leaves the domain.  Returns the number of walks that hit
 * the step cap (0 for a valid gradient).
 * ------------------------------------------------------------------------- */
int orc_labels(int W, int H, int D, const double *data, int *desc, int *asc, int nthreads) {
    grid_t G;
    grid_init(&G, W, H, D);
    int *P = (int *)malloc(sizeof(int) * ((size_t)G.V + G.E + G.F + G.T));
    int *PV = P, *PE = P + G.V, *PF = PE + G.E, *PT = PF + G.F;
    pair_all(&G, data, PV, PE, PF, PT, nthreads);
    ctx_t c;
    memset(&c, 0, sizeof(c));
    c.G = G;
    c.PV = PV; c.PE = PE; c.PF = PF; c.PT = PT;
    int bad = 0;
    for (int v = 0; v < G.V; v++) {
        int cur = v;
        long long steps = 0;
        while (PV[cur] != -1) {
            int a, b;
            edge_verts(&G, PV[cur], &a, &b);
            cur = a == cur ? b : a;
            if (++steps > G.V) {
                bad++;
                break;
            }
        }
        desc[v] = cur;
    }
    for (int t0 = 0; t0 < G.T; t0++) {
        int cur = t0, old, lab = -1;
        long long steps = 0;
        do {
            old = cur;
            int t = PT[cur];
            if (t == -1) {
                lab = cur;
                break;
            }
            if (PF[t] == -1 || PT[PF[t]] != t) break;
            int t1 = -1, t2 = -1;
            cell_tetra(&c, t, &t1, &t2);
            cur = t1 == cur ? t2 : t1;
            if (++steps > G.T) {
                bad++;
                break;
            }
        } while (cur != old && cur != -1);
        asc[t0] = lab;
    }
    free(P);
    return bad;
}

/* helpers for tests: cofaces of triangles in get_cell_tetra order (-1 when
 * absent) and endpoints of edges (higher id first) */
void orc_face_cofaces(int W, int H, int D, int n, const int *faces, int *out2) {
    ctx_t c;
    memset(&c, 0, sizeof(c));
    grid_init(&c.G, W, H, D);
    for (int i = 0; i < n; i++) {
        int x = -1, y = -1;
        cell_tetra(&c, faces[i], &x, &y);
        out2[2 * i] = x;
        out2[2 * i + 1] = y;
    }
}

void orc_tri_verts(int W, int H, int D, int n, const int *faces, int *out3) {
    grid_t G;
    grid_init(&G, W, H, D);
    for (int i = 0; i < n; i++) tri_verts(&G, faces[i], &out3[3 * i], &out3[3 * i + 1], &out3[3 * i + 2]);
}

void orc_edge_ids(int W, int H, int D, int n, const int *pairs, int *out) {
    grid_t G;
    grid_init(&G, W, H, D);
    for (int i = 0; i < n; i++) {
        int x, y, z, x1, y1, z1;
        coords(&G, pairs[2 * i], &x, &y, &z);
        coords(&G, pairs[2 * i + 1], &x1, &y1, &z1);
        out[i] = edge_id(&G, x, y, z, x1, y1, z1);
    }
}

void orc_edge_verts(int W, int H, int D, int n, const int *edges, int *out2) {
    grid_t G;
    grid_init(&G, W, H, D);
    for (int i = 0; i < n; i++) edge_verts(&G, edges[i], &out2[2 * i], &out2[2 * i + 1]);
}

/* Mismatch anchors of the learned proposal's features: mask[v] = 1 when some
 * cell whose componentwise-minimum vertex is v is critical in exactly one of
 * the two pairings (the same per-cell test as get_false_*, main_3d.cu:
 * 2492-2550, gathered per anchor vertex instead of listed). */
void orc_mismatch_anchors(int W, int H, int D, const int *PV, const int *PE, const int *PF, const int *PT,
                          const int *QV, const int *QE, const int *QF, const int *QT, unsigned char *mask) {
    grid_t G;
    grid_init(&G, W, H, D);
    for (int i = 0; i < G.V; i++) mask[i] = (unsigned char)xor_crit(PV[i], QV[i]);
    int vs[4];
    for (int e = 0; e < G.E; e++)
        if (xor_crit(PE[e], QE[e])) {
            edge_verts(&G, e, &vs[0], &vs[1]);
            mask[anchor_of(&G, vs, 2)] = 1;
        }
    for (int t = 0; t < G.F; t++)
        if (xor_crit(PF[t], QF[t])) {
            tri_verts(&G, t, &vs[0], &vs[1], &vs[2]);
            mask[anchor_of(&G, vs, 3)] = 1;
        }
    for (int t = 0; t < G.T; t++)
        if (xor_crit(PT[t], QT[t])) {
            tet_verts(&G, t, &vs[0], &vs[1], &vs[2], &vs[3]);
            mask[anchor_of(&G, vs, 4)] = 1;
        }
}

/* ---------------------------------------------------------------------------
 * Link components (no counterpart in the reference, which classifies cells by
 * the discrete gradient; this is the piecewise-linear reading of "min / max /
 * saddle from the lower and upper link").  The link of vertex v is the
 * subcomplex of its 14 stencil neighbours whose simplices span a simplex with
 * v.  The Freudenthal triangulation is a flag complex: any neighbours that are
 * pairwise adjacent span a simplex with v, so the link's edges are the
 * adjacent neighbour pairs and its triangles the adjacent triples.  Lower
 * (upper) link: the neighbours below (above) v in compare_vertices order
 * (main_3d.cu:1043-1049).  Per vertex: out[v] = (lower components) |
 * (upper components) << 4.  counts: [0] vertices with an empty lower link
 * (minima), [1] with an empty upper link (maxima), [2] with one lower and one
 * upper component (regular), [3] sum of (lower components - 1) over vertices
 * with at least two (join saddles, by multiplicity), [4] the same for upper
 * components (split saddles), [5] sum over vertices of 1 - chi(lower link),
 * which equals the Euler characteristic of the grid's solid box, 1 (every
 * edge, triangle and tetrahedron is counted once, at its highest vertex).
 * ------------------------------------------------------------------------- */
static int link_adj(int i, int j) {
    return i != j && is_dir(DIRS[i][0] - DIRS[j][0], DIRS[i][1] - DIRS[j][1], DIRS[i][2] - DIRS[j][2]);
}

void orc_link_classes(int W, int H, int D, const double *data, unsigned char *out, long long counts[6]) {
    grid_t G;
    grid_init(&G, W, H, D);
    for (int k = 0; k < 6; k++) counts[k] = 0;
    for (int v = 0; v < G.V; v++) {
        const int x = v % W, y = (v / W) % H, z = v / (W * H);
        int side[14]; /* -1 below, 1 above, 0 outside the grid */
        for (int i = 0; i < 14; i++) {
            const int nx = x + DIRS[i][0], ny = y + DIRS[i][1], nz = z + DIRS[i][2];
            if (nx < 0 || ny < 0 || nz < 0 || nx >= W || ny >= H || nz >= D) {
                side[i] = 0;
                continue;
            }
            const int n = nx + ny * W + nz * W * H;
            const int below = data[n] < data[v] || (data[n] == data[v] && n < v);
            side[i] = below ? -1 : 1;
        }
        int comps[2] = {0, 0};
        for (int h = 0; h < 2; h++) {
            const int want = h == 0 ? -1 : 1;
            int seen[14] = {0};
            for (int i = 0; i < 14; i++) {
                if (side[i] != want || seen[i]) continue;
                comps[h]++;
                int stack[14], sp = 0;
                stack[sp++] = i;
                seen[i] = 1;
                while (sp) {
                    const int a = stack[--sp];
                    for (int b = 0; b < 14; b++)
                        if (side[b] == want && !seen[b] && link_adj(a, b)) {
                            seen[b] = 1;
                            stack[sp++] = b;
                        }
                }
            }
        }
        long long nv = 0, ne = 0, nt = 0; /* the lower link's simplices */
        for (int i = 0; i < 14; i++) {
            if (side[i] != -1) continue;
            nv++;
            for (int j = i + 1; j < 14; j++) {
                if (side[j] != -1 || !link_adj(i, j)) continue;
                ne++;
                for (int k = j + 1; k < 14; k++)
                    if (side[k] == -1 && link_adj(i, k) && link_adj(j, k)) nt++;
            }
        }
        out[v] = (unsigned char)(comps[0] | (comps[1] << 4));
        if (comps[0] == 0) counts[0]++;
        if (comps[1] == 0) counts[1]++;
        if (comps[0] == 1 && comps[1] == 1) counts[2]++;
        if (comps[0] >= 2) counts[3] += comps[0] - 1;
        if (comps[1] >= 2) counts[4] += comps[1] - 1;
        counts[5] += 1 - (nv - ne + nt);
    }
}
