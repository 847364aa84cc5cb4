/*
 * dmtz.h — C ABI of libdmtz, the GB300 (sm_103a) implementation of DMTz's
 * topology-correction path for lossy-compressed 3-D scalar fields.
 *
 * The reference (main_3d.cu) has no library interface: its boundary is the
 * process (argv + files, main_3d.cu:6255-6393) and a set of device-global
 * kernels driven by a host loop.  Each entry point below replaces one stage
 * of that program; the comment on each names the reference code it stands
 * in for.  Plain pointers and sizes only; no CUDA or torch types.
 *
 * Conventions
 *   - Fields are float64, x fastest: value of vertex (x,y,z) at x + y*W + z*W*H
 *     (main_3d.cu:1945-1947).  W, H, D >= 2.
 *   - Pairing arrays use the reference's cell numbering (getEdgeID,
 *     getTriangleID, getTetrahedraID) and its union encoding: -1 = unpaired,
 *     otherwise the id of the partner cell of the next lower or higher
 *     dimension.  Cell counts: dmtz_cell_counts().
 *   - Pointers are host pointers unless on_device != 0, in which case they are
 *     device pointers on the context's device.
 *   - Every call returns a dmtz_status; dmtz_last_error() gives a message.
 *     The library never exits the process.  One context per host thread.
 */
#ifndef DMTZ_H
#define DMTZ_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    DMTZ_OK = 0,
    DMTZ_ERR_CUDA = 1,          /* a CUDA runtime call failed */
    DMTZ_ERR_ARG = 2,           /* invalid argument (dims, NaN/Inf input, bad flags) */
    DMTZ_ERR_IO = 3,            /* file read/write failed (CLI helpers) */
    DMTZ_ERR_NONCONVERGED = 4,  /* iteration cap reached before the complexes agree */
    DMTZ_ERR_CYCLE = 5,         /* a gradient path walk exceeded its step cap */
    DMTZ_ERR_BOUND = 6,         /* an output value violates the error bound */
    DMTZ_ERR_UNSUPPORTED = 7,   /* flag combination not implemented */
    DMTZ_ERR_OOB = 8,           /* the reference rules would index out of range here */
    DMTZ_ERR_TOO_LARGE = 9      /* grid exceeds the fixed scratch of dmtz_extract_noalloc, or a
                                   wall search outgrew its largest tier */
} dmtz_status;

typedef struct dmtz_ctx dmtz_ctx;

/* The reference's seven command-line flags (main_3d.cu:6265-6272) plus
 * controls of this implementation. */
typedef struct {
    int preserve_saddles;     /* argv[4] */
    int preserve_vpath;       /* argv[5] */
    int preserve_geometry;    /* argv[6] */
    int filtration;           /* argv[7] */
    int preserve_connectors;  /* argv[8]; 1 (with preserve_vpath = 1): wall checks of the
                                 original 2-saddles in the separatrix phase (see
                                 dmtz_wall_detect); such runs use the host-driven loop */
    int preserve_type;        /* argv[9] */
    int edit_type;            /* argv[10] */
    int max_rounds;           /* cap on fix/apply rounds; 0 = 100000 */
    int use_graph;            /* 1: run the loop as a CUDA graph with a device-side
                                 convergence flag; 0: host-driven loop */
    int break_stalls;         /* 1: when a round changes no value and no edit counter
                                 (a state the reference's loop repeats forever), set the
                                 values around the remaining mismatches back to the
                                 original ones (always within the bound) and go on;
                                 0: keep going until max_rounds, as the reference would.
                                 Rounds that make progress are the same either way. */
    int strict_separatrices;  /* 0: the reference's descending separatrix check
                                 (get_false_ds_vpath, main_3d.cu:4837-4959), which
                                 compares each 1-saddle endpoint's pairing at the first
                                 vertex of its path only; the output is the reference's.
                                 1 (geometry mode): the whole original descending path
                                 of every endpoint is compared, and its first differing
                                 vertex fixed with the same rule (fix_ds_vpath), so that
                                 every descending separatrix label agrees on exit; the
                                 output then differs from the reference's. */
} dmtz_opts;

typedef struct {
    int64_t outer_iterations;   /* total_ite of the reference (main_3d.cu:6786) */
    int64_t cp_rounds;          /* rounds of the critical-point loop */
    int64_t path_rounds;        /* rounds of the separatrix phase */
    int64_t initial_mismatch[4];/* min, 1-saddle, 2-saddle, max before correction */
    int64_t final_mismatch[4];
    int64_t final_paths[2];     /* ascending, descending separatrix records */
    int64_t edited_vertices;    /* vertices the correction wrote at least once (a
                                   vertex written back to its input value counts) */
    int32_t converged;
    int32_t error_flags;        /* bit 0: out-of-range index met by a fix rule,
                                   bit 1: path-walk step cap reached */
    double seconds;             /* device time of the whole correction (CUDA events
                                   on the context's stream, inputs already on the device) */
    int64_t kernel_launches;    /* kernels this call launched */
    double phase_ms[6];         /* device time per phase, as the reference's timers
                                   (main_3d.cu:6419-6436): gradient pairing + mismatch
                                   detection, critical-point fixes, separatrix detection,
                                   separatrix fixes, value update, set-up */
    int64_t stall_breaks;       /* rounds in which break_stalls reset values */
    int64_t final_walls;        /* wall records left (preserve_connectors = 1) */
} dmtz_report;

/* Context: owns the device, a stream and all scratch memory.
 * Replaces the device globals and cudaMalloc calls of main_3d.cu:43-129,
 * 6466-6714. */
dmtz_status dmtz_ctx_create(dmtz_ctx **out, int device);
void dmtz_ctx_destroy(dmtz_ctx *ctx);
const char *dmtz_last_error(const dmtz_ctx *ctx);

/* Cell counts V, E, F, T of a W x H x D grid (main_3d.cu:6401-6415). */
dmtz_status dmtz_cell_counts(int W, int H, int D, int64_t out[4]);

/* Discrete gradient of one field: the five pairing passes processVertices,
 * edgePairingKernel(a2=0), trianglePairingKernel(a2=0), edgePairingKernel(a2=1),
 * trianglePairingKernel(a2=1) (main_3d.cu:1930-2316), exported in the
 * reference's layout (paired_vertices / _edges / _faces / _tetrahedras). */
dmtz_status dmtz_extract(dmtz_ctx *ctx, int W, int H, int D, const double *data, int on_device,
                         int32_t *PV, int32_t *PE, int32_t *PF, int32_t *PT);

/* Critical-cell mismatch between the gradients of `orig` and `decp`
 * (get_false_minimum/saddle/2_saddle/maximum, main_3d.cu:2492-2550).
 * counts[4] = {min, 1-saddle, 2-saddle, max}; each list (capacity = the
 * number of cells of that dimension, may be NULL) receives the mismatched cell
 * ids in increasing order. */
dmtz_status dmtz_mismatch(dmtz_ctx *ctx, int W, int H, int D, const double *orig, const double *decp,
                          int64_t counts[4], int32_t *lmin, int32_t *lsad, int32_t *l2sad, int32_t *lmax);

/* One critical-point fix round (fix_minimum, fix_saddle, fix_2saddle,
 * fix_maximum; main_3d.cu:2554-4303) on the current mismatch: writes the
 * per-vertex delta that the reference's d_deltaBuffer would hold, or
 * -2000*range (the reference's "no request" sentinel) where nothing was
 * requested.  edit_counter: per-vertex delta_counter (host, V ints). */
dmtz_status dmtz_fix_round(dmtz_ctx *ctx, int W, int H, int D, const double *orig, const double *decp,
                           const int32_t *edit_counter, double rel_eps, int preserve_saddles, int edit_type,
                           double *delta_out);

/* Geometry-mode separatrix check (get_false_as_vpath + is_false,
 * get_false_ds_vpath; main_3d.cu:4437-4610, 4837-4959).  counts[2] =
 * {ascending, descending}; as_tet/as_cur: starting coface tet and the tet
 * where the pairing first differs; ds_edge/ds_vert: 1-saddle and vertex.
 * Lists are sorted by (first, second); capacities F (ascending), E
 * (descending). */
dmtz_status dmtz_path_detect(dmtz_ctx *ctx, int W, int H, int D, const double *orig, const double *decp,
                             int64_t counts[2], int32_t *as_tet, int32_t *as_cur, int32_t *ds_edge,
                             int32_t *ds_vert);

/* dmtz_path_detect with the descending half of strict_separatrices = 1: a
 * record is the first vertex on a 1-saddle endpoint's whole original
 * descending path whose decompressed pairing differs (no counterpart in the
 * reference, whose walk stops after the first vertex).  Same arguments. */
dmtz_status dmtz_path_detect_strict(dmtz_ctx *ctx, int W, int H, int D, const double *orig, const double *decp,
                                    int64_t counts[2], int32_t *as_tet, int32_t *as_cur, int32_t *ds_edge,
                                    int32_t *ds_vert);

/* Connectivity-mode separatrix check (preserve_vpath=1, preserve_geometry=0):
 * a separatrix is false when its end differs, not its geometry.  Descending
 * half as get_false_ds_vpath_connectivity (main_3d.cu:4961-5062; ds_vert is
 * the reference's trouble maker, -1 when none was met).  Ascending half as
 * get_false_as_vpath_connectivity (main_3d.cu:4761-4835) meant it: the
 * original ends are kept per triangle, where the reference indexes them by a
 * loop counter shared by all triangles (a race, so its own output depends on
 * scheduling).  Same arguments and record layout as dmtz_path_detect. */
dmtz_status dmtz_path_detect_connectivity(dmtz_ctx *ctx, int W, int H, int D, const double *orig,
                                          const double *decp, int64_t counts[2], int32_t *as_tet, int32_t *as_cur,
                                          int32_t *ds_edge, int32_t *ds_vert);

/* Wall check of preserve_connectors = 1.  Replaces get_false_ds_wall
 * (main_3d.cu:5064-5121), restated without its races (shared per-block stack,
 * shared spill buffer, visited marks shared by all 2-saddles, record-index
 * array aliasing the record array, launch covering only the first V faces):
 * every original 2-saddle face runs its own depth-first search, in the
 * reference's order, over the faces its original V-paths reach, and records
 * the first edge whose original and decompressed pairings differ.
 * count: records; w_sad / w_edge (capacity: the number of original
 * 2-saddles, or the number of triangles) receive (2-saddle face, edge) pairs
 * sorted by face.  Either array may be null. */
dmtz_status dmtz_wall_detect(dmtz_ctx *ctx, int W, int H, int D, const double *orig, const double *decp,
                             int64_t *count, int32_t *w_sad, int32_t *w_edge);

/* The whole correction (main_3d.cu:6255-7149): extracts both complexes and
 * edits `decp` in place until they agree.  bound = (max(orig) - min(orig)) *
 * rel_eps, as in the reference.  edit_counter_out (optional, V ints) receives
 * delta_counter.  Returns DMTZ_ERR_NONCONVERGED if opts->max_rounds is hit. */
dmtz_status dmtz_correct(dmtz_ctx *ctx, int W, int H, int D, const double *orig, double *decp, int on_device,
                         double rel_eps, const dmtz_opts *opts, dmtz_report *report, int32_t *edit_counter_out);

/* Manifold labels of one field's discrete gradient (no reference kernel
 * materialises them; they follow the reference's own path rules):
 *   desc[v] (V ints): the minimum reached from vertex v by repeatedly moving
 *     to the other endpoint of its paired edge (processVertices pairing);
 *   asc[t] (T ints): the maximum tetrahedron reached from tetrahedron t by
 *     the ascending walk of is_false (main_3d.cu:4437-4497: paired facet, then
 *     that facet's other coface), or -1 when the walk leaves the domain.
 * Separatrix labels are these labels at the endpoints of 1-saddle edges and
 * at the cofaces of 2-saddle triangles.  Returns DMTZ_ERR_CYCLE if pointer
 * jumping does not settle in 64 rounds. */
dmtz_status dmtz_labels(dmtz_ctx *ctx, int W, int H, int D, const double *data, int on_device, int32_t *desc,
                        int32_t *asc);

/* Separatrix agreement of `decp`'s gradient with `orig`'s (the acceptance
 * check "the re-extracted MSC has the original's separatrix labels"; no
 * reference counterpart): out[0] = endpoints of original 1-saddle edges
 * compared, out[1] = of those, endpoints whose descending label (as
 * dmtz_labels) is the same in both fields; out[2] = cofaces of original
 * 2-saddle triangles compared, out[3] = of those, cofaces with the same
 * ascending label; out[4] = cells whose criticality differs (all four
 * dimensions).  Labels and counts are computed on the device. */
dmtz_status dmtz_separatrix_agreement(dmtz_ctx *ctx, int W, int H, int D, const double *orig, const double *decp,
                                      int on_device, int64_t out[5]);

/* Piecewise-linear classification of every vertex by its link (no
 * counterpart in the reference, whose critical cells are the unpaired cells
 * of the discrete gradient; a diagnostic).  The link of v is spanned by its
 * 14 stencil neighbours (two are joined when they are adjacent: the
 * triangulation is a flag complex); its lower (upper) part holds the
 * neighbours below (above) v in the reference's (value, id) order.
 * out (host, V bytes, may be NULL): lower components | upper components << 4.
 * counts: [0] minima (empty lower link; the same vertices the reference
 * leaves unpaired), [1] maxima (empty upper link), [2] regular (one lower and
 * one upper component), [3] join-saddle multiplicity (sum of lower
 * components - 1 where there are two or more), [4] split-saddle multiplicity
 * (the same for upper components), [5] sum over vertices of 1 - chi(lower
 * link), the Euler characteristic of the grid's box: always 1. */
dmtz_status dmtz_link_classes(dmtz_ctx *ctx, int W, int H, int D, const double *data, int on_device, uint8_t *out,
                              int64_t counts[6]);

/* Decompression model on the GPU, for benchmarks and training data (the
 * reference runs an external compressor and reads the result back,
 * main_3d.cu:6331-6356): decp = SZ-style error-bounded quantisation of orig,
 * fmin + 2 eps * rint((orig - fmin) / (2 eps)) with eps = rel_eps x range,
 * plus uniform noise in [-eps, eps) on a fraction noise_frac of the vertices
 * (a counter-based hash of seed and vertex: the same output for the same
 * inputs on any GPU), clamped into [orig - eps, orig + eps]. */
dmtz_status dmtz_quantize(dmtz_ctx *ctx, int W, int H, int D, const double *orig, double *decp, int on_device,
                          double rel_eps, double noise_frac, uint64_t seed);

/* ---- batching and tuning (no counterpart in the reference, which corrects
 * one field per process run) ---- */

enum { DMTZ_F64 = 0, DMTZ_F32 = 1 };

/* One field of a batch, in host memory.  orig/decp hold W*H*D values of
 * `dtype`; float32 input is widened to float64 (exactly) and corrected in
 * float64, as the reference would correct the widened file.  out receives
 * the corrected field (W*H*D doubles). */
typedef struct {
    int W, H, D;
    int dtype;
    const void *orig;
    const void *decp;
    double *out;
    double rel_eps;
} dmtz_instance;

/* Correct n fields of any sizes.  `workers` contexts (default 8), each with
 * its own stream and buffers, take fields from a shared queue and run the
 * correction (with opts->use_graph, as a device-driven graph); their kernels
 * overlap on the GPU.  reports[i] / status[i] (optional) per field; returns
 * the first failing status or DMTZ_OK. */
dmtz_status dmtz_correct_batch(dmtz_ctx *ctx, int n, const dmtz_instance *inst, const dmtz_opts *opts,
                               dmtz_report *reports, dmtz_status *status, int workers);

/* Brick shape (0: 8x4x4, 1: 16x4x2, 2: 32x2x2 anchors) and blocks per SM of
 * the gradient sweeps.  Results do not depend on them, only speed.
 * dmtz_autotune times a full sweep of `decp` for every shape and 8, 16, 32, 64
 * blocks per SM, keeps the fastest in the context and returns it in best[2]. */
dmtz_status dmtz_set_tuning(dmtz_ctx *ctx, int shape, int blocks_per_sm);
/* Memory of the mismatch lists (critical cells that differ between the two
 * gradients).  Each of the four lists starts with room for `fraction` of the
 * cells of its dimension, at least `min_entries` (defaults 1/16 and 2^20),
 * and grows when a round produces more mismatches; results never depend on
 * it.  The separatrix records are sized from the original field's saddle
 * counts.  Together this keeps a correction near 125 bytes of device memory
 * per vertex, so a 1024^3 field fits on one GPU. */
dmtz_status dmtz_set_list_reserve(dmtz_ctx *ctx, double fraction, int64_t min_entries);
/* name of the context's device (for keying tuning caches) */
dmtz_status dmtz_device_name(const dmtz_ctx *ctx, char *buf, int len);
dmtz_status dmtz_get_tuning(const dmtz_ctx *ctx, int *shape, int *blocks_per_sm);
dmtz_status dmtz_autotune(dmtz_ctx *ctx, int W, int H, int D, const double *orig, const double *decp, int on_device,
                          int best[2], double *best_ms);

/* Timing of the gradient sweep that every correction round runs (the five
 * pairing passes of main_3d.cu:6864-6874 plus the critical-cell comparison
 * of :6903-6909), `reps` times on the context's stream between CUDA events.
 * ms[0..5] = mean per-launch time of the vertex, edge, triangle, edge,
 * triangle and criticality kernels; ms[6] = mean time of one whole sweep.
 * No counterpart call in the reference (measurement only). */
dmtz_status dmtz_profile_sweep(dmtz_ctx *ctx, int W, int H, int D, const double *orig, const double *decp,
                               int on_device, int reps, double ms[7]);

/* ---- learned proposal (no counterpart in the reference) ----
 * A small convolutional network proposes corrected values near mismatches;
 * the exact correction loop then starts from that proposal instead of the
 * decompressed field.  Network: 3x3x3 convolutions 16 -> 32 -> 32 -> 32 -> 1
 * channels, ReLU between layers, bf16 weights and activations with fp32
 * accumulation on the tensor cores.  At an active vertex the proposal
 * p = f + bound * tanh(o) replaces g where it lowers g by at least
 * min_drop * bound (dmtz_cnn_set_min_drop, default 0.5); values stay within
 * the bound.
 *
 * Features (dmtz_features): per vertex 16 bf16 channels, channels-last:
 *   0 (g - f) / bound; 1 = 1 where the vertex's own cells differ in
 *   criticality between the two gradients; 2..15 tanh((f(u) - f(v)) /
 *   (4 bound)) for the 14 Freudenthal neighbours u (0 outside the grid).
 * active[v] = 1 within 2 vertices (per axis) of such a mismatch.
 *
 * Network buffers (feat, out, target, active) are DEVICE pointers on the
 * network's device; feat must be 16-byte aligned.  Calls are synchronous. */
typedef struct dmtz_cnn dmtz_cnn;
#define DMTZ_CNN_FEATURES 16
/* number of float parameters (get/set/grad layout: per layer, weights
 * [27 taps][out][in] (tap = (dz+1)*9 + (dy+1)*3 + dx+1), then bias [out];
 * layers 16->32, 32->32, 32->32, 32->16 of which only output 0 is used) */
int64_t dmtz_cnn_num_params(void);
dmtz_status dmtz_cnn_create(dmtz_cnn **out, int device, uint64_t seed);
void dmtz_cnn_destroy(dmtz_cnn *net);
const char *dmtz_cnn_last_error(const dmtz_cnn *net);
dmtz_status dmtz_cnn_set_params(dmtz_cnn *net, const float *host);  /* also resets Adam */
dmtz_status dmtz_cnn_get_params(dmtz_cnn *net, float *host);
dmtz_status dmtz_cnn_get_grads(dmtz_cnn *net, float *host);
/* out (V floats) = pre-tanh output o; train != 0 keeps the activations for
 * dmtz_cnn_backward */
dmtz_status dmtz_cnn_forward(dmtz_cnn *net, int W, int H, int D, const void *feat, float *out, int train);
/* loss = sum_v w_v (tanh(o_v) - target_v)^2 / sum_v w_v with the weight
 * w_v = active[v] (0..255; a 0/1 mask gives the mean over active vertices);
 * the parameter gradient of that loss goes into the network's gradient
 * buffer */
dmtz_status dmtz_cnn_backward(dmtz_cnn *net, int W, int H, int D, const float *target, const uint8_t *active,
                              double *loss);
/* Tensor-core path of the convolutions (no counterpart in the reference):
 * 1 = tcgen05.mma with the accumulators in tensor memory,
 * 2 (the default) = tcgen05.mma with the three x-taps of each (y, z) offset in one product
 * of three times the width (partial sums shifted and added in the epilogue),
 * 0 = the warp-level mma.sync kernels.  Same arithmetic (bf16 products, f32
 * sums); results differ only in the order of the f32 sums. */
dmtz_status dmtz_cnn_set_tensor_path(dmtz_cnn *net, int path);
/* Measurement only: the tensor pipe's rate, in TFLOP/s over all SMs, for
 * back-to-back tcgen05.mma of shape M = 128, N = n (32, 48, 64, 96, 128 or
 * 256), K = 16 (bf16, f32 accumulators), `reps` x 8 per SM.  The
 * convolutions' products have N = 32 on tensor path 1 and N = 96 (three taps
 * of 32 output channels) on path 2: those rates bound them. */
dmtz_status dmtz_cnn_mma_ceiling(dmtz_cnn *net, int n, int reps, double *tflops);
/* proposal threshold in units of the bound, 0..2 */
dmtz_status dmtz_cnn_set_min_drop(dmtz_cnn *net, float min_drop);
/* one Adam step (beta 0.9 / 0.999, eps 1e-8) with learning rate lr */
dmtz_status dmtz_cnn_step(dmtz_cnn *net, float lr);
/* Timing of the network kernels on a W x H x D grid (CUDA events on the
 * network's stream, `reps` repetitions each; measurement only): ms[0] = one
 * forward pass (inference), ms[1] = one training step (forward, backward,
 * Adam with learning rate 0; parameters and Adam state are restored
 * afterwards), ms[2] = one
 * 32 -> 32 convolution launch, ms[3] = one 32 x 32 weight-gradient launch
 * (with its reduction). */
dmtz_status dmtz_cnn_profile(dmtz_cnn *net, int W, int H, int D, const void *feat, float *out, const float *target,
                             const uint8_t *active, int reps, double ms[4]);
/* features and active mask of (orig, decp); feat / active are device
 * pointers (V x 16 bf16, V bytes); orig / decp as in dmtz_correct */
dmtz_status dmtz_features(dmtz_ctx *ctx, int W, int H, int D, const double *orig, const double *decp, int on_device,
                          double rel_eps, void *feat, uint8_t *active);
/* dmtz_correct started from the network's proposal.  The result keeps the
 * reference loop's guarantees (gradients agree, |decp - orig| <= bound) but
 * is not the reference's output, which starts from the unedited field.
 * report->seconds includes features, network and proposal (phase "set-up"). */
dmtz_status dmtz_correct_learned(dmtz_ctx *ctx, dmtz_cnn *net, int W, int H, int D, const double *orig,
                                 double *decp, int on_device, double rel_eps, const dmtz_opts *opts,
                                 dmtz_report *report, int32_t *edit_counter_out);

/* Allocation-free variant of dmtz_extract, for callers that cannot call
 * cudaMalloc: applications whose device memory is owned by their own pool
 * allocator (which forbids or cannot account for foreign allocations), and
 * latency-sensitive pipelines where a cudaMalloc/cudaFree would synchronise
 * the device in the middle of their stream work.  It has no counterpart in
 * the reference.
 *
 * The caller passes every buffer: `data` (V doubles) and the four output
 * arrays (dmtz_cell_counts sizes, int32), all DEVICE pointers on the current
 * device, and a cudaStream_t as `stream` (NULL = the legacy default stream).
 * The call only enqueues kernels on that stream and returns; results are
 * ready when the stream reaches that point.  Inputs must be finite (not
 * checked here).
 *
 * Scratch: the per-vertex gradient state lives in one fixed device array
 * inside the library, sized for at most DMTZ_NOALLOC_MAX_VERTICES vertices
 * (64^3; about 7.6 MB that every GPU which loads the library keeps until the
 * process exits).  Larger grids return DMTZ_ERR_TOO_LARGE.  The first call on
 * a device looks up that array's device address (cudaGetSymbolAddress), so
 * make that first call before any stream capture.  The address is kept for
 * the life of the process: a cudaDeviceReset between calls is not supported.
 * A CUDA error already pending when the call starts is returned as
 * DMTZ_ERR_CUDA and left pending; nothing is launched then.  All calls share the one
 * array: calls that can overlap on the GPU (different streams, or different
 * host threads) race and must be serialised by the caller. */
#define DMTZ_NOALLOC_MAX_VERTICES (64 * 64 * 64)
dmtz_status dmtz_extract_noalloc(int W, int H, int D, const double *data, int32_t *PV, int32_t *PE, int32_t *PF,
                                 int32_t *PT, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* DMTZ_H */
