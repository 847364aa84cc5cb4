/*
 * dmtz_oracle.h — CPU oracle for the DMTz topology-correction path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a serial C restatement of the
 * reference's CUDA kernels (main_3d.cu), used by tests/, by the smoke check
 * and by bench.py's CPU-baseline leg to check and to time the product.  The
 * product library (dmtz_gb300/) never links, loads or calls it.
 *
 * Pinning: the oracle is checked against outputs of the reference program
 * itself (built from main_3d.cu with its one-character compile fix and run
 * on a GB300); the fixtures live in tests/golden/ together with the script
 * that produced them (oracle/ref_harness.py).
 *
 * Conventions follow the reference exactly: vertex id = x + y*W + z*W*H,
 * edge/face/tet ids as produced by getEdgeID / getTriangleID /
 * getTetrahedraID, pairing arrays hold -1 for "unpaired" and otherwise the
 * id of the partner cell (a union of lower/higher dimension, disambiguated by
 * back-pointer checks), all ids are 32-bit ints.
 */
#ifndef DMTZ_ORACLE_H
#define DMTZ_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* counts of cells of the implicit Freudenthal complex (main_3d.cu:6401-6415) */
void orc_counts(int W, int H, int D, long long out[4]);

/* Five-pass discrete-gradient pairing of one field (main_3d.cu:1930-2316).
 * Arrays are overwritten (all -1 first, as init_* do).  Returns number of
 * out-of-bounds index events (0 for any valid grid). */
int orc_pair(int W, int H, int D, const double *data,
             int *PV, int *PE, int *PF, int *PT, int nthreads);

/* Critical-cell mismatch counts between two pairings (get_false_*,
 * main_3d.cu:2492-2550).  Lists (optional, may be NULL) receive the cell ids
 * in increasing id order. counts = {min, saddle, 2saddle, max}. */
void orc_cp_mismatch(int W, int H, int D,
                     const int *PV, const int *PE, const int *PF, const int *PT,
                     const int *QV, const int *QE, const int *QF, const int *QT,
                     int counts[4], int *lmin, int *lsad, int *l2sad, int *lmax);

/* One critical-point fix round (fix_minimum / fix_saddle / fix_2saddle /
 * fix_maximum, main_3d.cu:2554-4303) on the given mismatch lists.  buf is the
 * per-vertex delta buffer (V doubles) initialised by the caller to the
 * sentinel -2000*range; cnt the per-vertex edit counter.  Returns the number
 * of out-of-bounds events. */
int orc_fix_cp(int W, int H, int D, const double *f, const double *g,
               const int *cnt, double bound, double range, int edit_type,
               int preserve_saddles,
               const int *PV, const int *PE, const int *PF, const int *PT,
               const int *QV, const int *QE, const int *QF, const int *QT,
               const int counts[4], const int *lmin, const int *lsad,
               const int *l2sad, const int *lmax, double *buf);

/* Geometry-mode separatrix detection (get_false_as_vpath + is_false,
 * get_false_ds_vpath; main_3d.cu:4437-4610, 4837-4959).  Outputs the record
 * lists in increasing saddle-id order: as_tet[k] = starting coface tet,
 * as_cur[k] = tet where the pairing first differs; ds_edge[k] = 1-saddle,
 * ds_vert[k] = vertex where the pairing differs.  counts = {as, ds}.
 * Returns number of out-of-bounds/cycle events. */
int orc_path_detect(int W, int H, int D,
                    const int *PV, const int *PE, const int *PF, const int *PT,
                    const int *QV, const int *QE, const int *QF, const int *QT,
                    int counts[2], int *as_tet, int *as_cur,
                    int *ds_edge, int *ds_vert);

/* Full correction run (host loop main_3d.cu:6255-7149).
 *   f, g       : original / decompressed field (g is corrected in place)
 *   rel_eps    : the relative error bound argument
 *   flags[7]   : preserve_saddles, preserve_vpath, preserve_geometry,
 *                filtration, preserve_connectors, preserve_type, edit_type
 *   max_outer  : cap on outer iterations (0 = 100000)
 *   stats[8]   : out: outer iterations (total_ite), CP inner iterations,
 *                out-of-bounds events, converged(1/0), initial mismatch
 *                counts min, saddle, 2saddle, max
 *   cnt_out    : out (optional): final per-vertex edit counter
 * preserve_connectors=1 runs the wall checks of orc_wall_detect in the
 * separatrix phase (with preserve_vpath=1).  Returns 0. */
int orc_correct(int W, int H, int D, const double *f, double *g,
                double rel_eps, const int flags[7], int max_outer,
                int nthreads, long long stats[8], int *cnt_out);
/* id helpers: descending vertex triples of faces; edge ids of vertex pairs */
void orc_tri_verts(int W, int H, int D, int n, const int *faces, int *out3);
void orc_edge_ids(int W, int H, int D, int n, const int *pairs, int *out);
/* Walls of the original 2-saddles (get_false_ds_wall without its races):
 * per 2-saddle face, its own depth-first search over faces reachable by
 * original V-paths; the first edge whose original and decompressed pairings
 * differ is the record (w_sad[k], w_edge[k]); *count records, pops = stack
 * pops of all searches.  Returns the number of out-of-range reads. */
int orc_wall_detect(int W, int H, int D, const int *PV, const int *PE, const int *PF, const int *PT, const int *QV,
                    const int *QE, const int *QF, const int *QT, int *count, int *w_sad, int *w_edge,
                    long long *pops);
/* 1: the descending separatrix checks of orc_path_detect and of the
 * correction loops walk each 1-saddle endpoint's whole original descending
 * path and record its first vertex whose decompressed pairing differs (the
 * reference's get_false_ds_vpath compares the first vertex only); 0 (the
 * default): the reference's check. */
void orc_set_strict_ds(int on);
/* orc_correct with stall breaking (break_stalls = 1: a round that changes no
 * value and no edit counter resets a box around the remaining mismatches to
 * the original values; stats[8] = such breaks). */
int orc_correct_ex(int W, int H, int D, const double *f, double *g, double rel_eps, const int flags[7],
                   int max_outer, int nthreads, int break_stalls, long long stats[9], int *cnt_out);
/* orc_correct_ex with an explicit cap on fix/apply rounds (max_rounds > 0;
 * otherwise 64 x max_outer): the state after exactly max_rounds rounds of a
 * loop that does not converge is the reference's after the same rounds. */
int orc_correct_rounds(int W, int H, int D, const double *f, double *g, double rel_eps, const int flags[7],
                       int max_outer, long long max_rounds, int nthreads, int break_stalls, long long stats[9],
                       int *cnt_out);

/* Manifold labels: desc[v] = minimum reached along the steepest-descent
 * pairing, asc[t] = maximum reached by the ascending tetrahedron walk, -1 if
 * it leaves the domain.  Returns the number of walks that hit the step cap. */
int orc_labels(int W, int H, int D, const double *data, int *desc, int *asc, int nthreads);

/* cofaces of triangles (get_cell_tetra order, -1 when absent) and edge
 * endpoints (higher id first), two ints per input id */
void orc_face_cofaces(int W, int H, int D, int n, const int *faces, int *out2);
void orc_edge_verts(int W, int H, int D, int n, const int *edges, int *out2);

/* Connectivity-mode separatrix check (preserve_vpath=1, preserve_geometry=0;
 * get_false_as_vpath_connectivity with the intended per-triangle index and
 * get_false_ds_vpath_connectivity, main_3d.cu:4613-4835, 4961-5062): records
 * as orc_path_detect's, ds_vert = the trouble maker (may be -1).  Returns the
 * number of out-of-bounds events. */
int orc_path_detect_conn(int W, int H, int D,
                         const int *PV, const int *PE, const int *PF, const int *PT,
                         const int *QV, const int *QE, const int *QF, const int *QT,
                         int counts[2], int *as_tet, int *as_cur, int *ds_edge, int *ds_vert);

/* mask[v] (V bytes) = 1 when a cell anchored at v (componentwise-minimum
 * vertex) is critical in exactly one of the two pairings */
void orc_mismatch_anchors(int W, int H, int D,
                          const int *PV, const int *PE, const int *PF, const int *PT,
                          const int *QV, const int *QE, const int *QF, const int *QT, unsigned char *mask);

/* Link components of every vertex (lower | upper << 4) and their summary
 * counts: minima, maxima, regular, join-saddle and split-saddle
 * multiplicities, and sum(1 - chi(lower link)) (= 1). */
void orc_link_classes(int W, int H, int D, const double *data, unsigned char *out, long long counts[6]);

#ifdef __cplusplus
}
#endif
#endif
