"""ctypes front end of the CPU oracle (test infrastructure only).

Only tests/, the smoke check and bench.py's CPU-baseline leg import this
module; the product package never does.  The oracle restates the reference
kernels of main_3d.cu serially in C (oracle/dmtz_oracle.c); arrays use the
reference's cell numbering and its -1 = "unpaired" convention.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libdmtz_oracle.so")
_lib = None

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")


def build() -> str:
    """Compile the oracle with its Makefile (idempotent)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        src = os.path.join(_HERE, "dmtz_oracle.c")
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        L.orc_counts.argtypes = [ctypes.c_int] * 3 + [_i64p]
        L.orc_pair.argtypes = [ctypes.c_int] * 3 + [_f64p, _i32p, _i32p, _i32p, _i32p, ctypes.c_int]
        L.orc_pair.restype = ctypes.c_int
        L.orc_cp_mismatch.argtypes = [ctypes.c_int] * 3 + [_i32p] * 8 + [_i32p] + [_i32p] * 4
        L.orc_fix_cp.argtypes = (
            [ctypes.c_int] * 3 + [_f64p, _f64p, _i32p, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int]
            + [_i32p] * 8 + [_i32p] + [_i32p] * 4 + [_f64p]
        )
        L.orc_fix_cp.restype = ctypes.c_int
        L.orc_path_detect.argtypes = [ctypes.c_int] * 3 + [_i32p] * 8 + [_i32p] + [_i32p] * 4
        L.orc_path_detect.restype = ctypes.c_int
        L.orc_path_detect_conn.argtypes = [ctypes.c_int] * 3 + [_i32p] * 8 + [_i32p] + [_i32p] * 4
        L.orc_path_detect_conn.restype = ctypes.c_int
        L.orc_link_classes.argtypes = [ctypes.c_int] * 3 + [_f64p, np.ctypeslib.ndpointer(dtype=np.uint8,
                                                                                         flags="C_CONTIGUOUS"), _i64p]
        L.orc_link_classes.restype = None
        L.orc_set_strict_ds.argtypes = [ctypes.c_int]
        L.orc_set_strict_ds.restype = None
        L.orc_correct.argtypes = [ctypes.c_int] * 3 + [_f64p, _f64p, ctypes.c_double, _i32p, ctypes.c_int,
                                                        ctypes.c_int, _i64p, _i32p]
        L.orc_correct.restype = ctypes.c_int
        L.orc_correct_ex.argtypes = [ctypes.c_int] * 3 + [_f64p, _f64p, ctypes.c_double, _i32p, ctypes.c_int,
                                                           ctypes.c_int, ctypes.c_int, _i64p, _i32p]
        L.orc_correct_ex.restype = ctypes.c_int
        L.orc_correct_rounds.argtypes = [ctypes.c_int] * 3 + [_f64p, _f64p, ctypes.c_double, _i32p, ctypes.c_int,
                                                               ctypes.c_longlong, ctypes.c_int, ctypes.c_int, _i64p,
                                                               _i32p]
        L.orc_correct_rounds.restype = ctypes.c_int
        L.orc_tri_verts.argtypes = [ctypes.c_int] * 4 + [_i32p, _i32p]
        L.orc_edge_ids.argtypes = [ctypes.c_int] * 4 + [_i32p, _i32p]
        L.orc_wall_detect.argtypes = [ctypes.c_int] * 3 + [_i32p] * 8 + [_i32p, _i32p, _i32p, _i64p]
        L.orc_wall_detect.restype = ctypes.c_int
        L.orc_labels.argtypes = [ctypes.c_int] * 3 + [_f64p, _i32p, _i32p, ctypes.c_int]
        L.orc_labels.restype = ctypes.c_int
        L.orc_face_cofaces.argtypes = [ctypes.c_int] * 4 + [_i32p, _i32p]
        L.orc_edge_verts.argtypes = [ctypes.c_int] * 4 + [_i32p, _i32p]
        L.orc_mismatch_anchors.argtypes = [ctypes.c_int] * 3 + [_i32p] * 8 + [
            np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")]
        L.orc_mismatch_anchors.restype = None
        _lib = L
    return _lib


def counts(dims):
    W, H, D = dims
    out = np.zeros(4, np.int64)
    lib().orc_counts(W, H, D, out)
    return tuple(int(v) for v in out)


def pair(data: np.ndarray, dims, threads: int = 1):
    """Five-pass gradient pairing -> (PV, PE, PF, PT) int32 arrays."""
    W, H, D = dims
    V, E, F, T = counts(dims)
    d = np.ascontiguousarray(data, dtype=np.float64).reshape(-1)
    assert d.size == V
    PV = np.empty(V, np.int32)
    PE = np.empty(E, np.int32)
    PF = np.empty(F, np.int32)
    PT = np.empty(T, np.int32)
    oob = lib().orc_pair(W, H, D, d, PV, PE, PF, PT, threads)
    if oob:
        raise RuntimeError(f"oracle pairing touched {oob} out-of-range ids")
    return PV, PE, PF, PT


def cp_mismatch(P, Q, dims):
    """Critical-cell mismatch lists (min, 1-saddle, 2-saddle, max)."""
    W, H, D = dims
    V, E, F, T = counts(dims)
    c = np.zeros(4, np.int32)
    lists = [np.empty(max(n, 1), np.int32) for n in (V, E, F, T)]
    lib().orc_cp_mismatch(W, H, D, *P, *Q, c, *lists)
    return [lists[k][: int(c[k])].copy() for k in range(4)]


def fix_cp(f, g, cnt, bound, rng, edit_type, preserve_saddles, P, Q, lists, dims):
    """One critical-point fix round -> per-vertex delta buffer (sentinel = -2000*range)."""
    W, H, D = dims
    V = counts(dims)[0]
    buf = np.full(V, -2000.0 * rng, np.float64)
    c = np.array([len(x) for x in lists], np.int32)
    ls = [np.ascontiguousarray(x, np.int32) if len(x) else np.zeros(1, np.int32) for x in lists]
    oob = lib().orc_fix_cp(W, H, D, np.ascontiguousarray(f, np.float64).reshape(-1),
                           np.ascontiguousarray(g, np.float64).reshape(-1), np.ascontiguousarray(cnt, np.int32),
                           float(bound), float(rng), int(edit_type), int(preserve_saddles), *P, *Q, c, *ls, buf)
    return buf, oob


def path_detect(P, Q, dims, connectivity=False, strict=False):
    """Separatrix records (as_tet, as_cur, ds_edge, ds_vert, oob) of geometry
    mode, or of connectivity mode (ds_vert = trouble maker).  strict: the
    descending records come from whole-path walks (not the reference's check)."""
    W, H, D = dims
    V, E, F, T = counts(dims)
    c = np.zeros(2, np.int32)
    a_t = np.empty(F, np.int32)
    a_c = np.empty(F, np.int32)
    d_e = np.empty(E, np.int32)
    d_v = np.empty(E, np.int32)
    fn = lib().orc_path_detect_conn if connectivity else lib().orc_path_detect
    lib().orc_set_strict_ds(int(bool(strict)))
    try:
        oob = fn(W, H, D, *P, *Q, c, a_t, a_c, d_e, d_v)
    finally:
        lib().orc_set_strict_ds(0)
    na, nd = int(c[0]), int(c[1])
    return a_t[:na].copy(), a_c[:na].copy(), d_e[:nd].copy(), d_v[:nd].copy(), oob


def correct(f, g, dims, rel_eps, flags, max_outer=0, threads=1, break_stalls=False, max_rounds=0, strict=False):
    """Run the full correction loop.  Returns (corrected g, stats dict, cnt).
    break_stalls: reset a box around the remaining mismatches to the original
    values when a round changes nothing (not in the reference, whose loop
    repeats such a round forever); stats["stall_breaks"] counts them.
    max_rounds > 0 caps the fix/apply rounds exactly (else 64 x max_outer).
    strict: whole-path descending separatrix checks (not the reference's)."""
    W, H, D = dims
    V = counts(dims)[0]
    ff = np.ascontiguousarray(f, np.float64).reshape(-1)
    gg = np.array(g, np.float64).reshape(-1)
    assert ff.size == V and gg.size == V
    fl = np.ascontiguousarray(flags, np.int32)
    st = np.zeros(9, np.int64)
    cnt = np.empty(V, np.int32)
    lib().orc_set_strict_ds(int(bool(strict)))
    try:
        rc = lib().orc_correct_rounds(W, H, D, ff, gg, float(rel_eps), fl, int(max_outer), int(max_rounds),
                                      int(threads), int(bool(break_stalls)), st, cnt)
    finally:
        lib().orc_set_strict_ds(0)
    if rc != 0:
        raise ValueError(f"oracle correction failed ({rc})")
    stats = dict(outer_iterations=int(st[0]), cp_iterations=int(st[1]), oob=int(st[2]), converged=bool(st[3]),
                 initial_mismatch=[int(x) for x in st[4:8]], stall_breaks=int(st[8]))
    return gg, stats, cnt


def tri_verts(faces, dims):
    """Descending vertex triples of faces -> (n, 3) int32."""
    f = np.ascontiguousarray(faces, np.int32)
    out = np.empty((max(f.size, 1), 3), np.int32)
    lib().orc_tri_verts(*dims, int(f.size), f if f.size else np.zeros(1, np.int32), out)
    return out[: f.size]


def edge_ids(pairs, dims):
    """Edge ids of adjacent vertex pairs ((n, 2) array)."""
    p = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
    out = np.empty(max(len(p), 1), np.int32)
    lib().orc_edge_ids(*dims, len(p), p if len(p) else np.zeros((1, 2), np.int32), out)
    return out[: len(p)]


def wall_detect(P, Q, dims):
    """Wall records of the original 2-saddles: (saddle faces, record edges,
    stack pops of all searches, out-of-range reads)."""
    W, H, D = dims
    V, E, F, T = counts(dims)
    c = np.zeros(1, np.int32)
    ws, we = np.empty(max(F, 1), np.int32), np.empty(max(F, 1), np.int32)
    pops = np.zeros(1, np.int64)
    oob = lib().orc_wall_detect(W, H, D, *P, *Q, c, ws, we, pops)
    n = int(c[0])
    return ws[:n].copy(), we[:n].copy(), int(pops[0]), oob


def labels(data, dims, threads: int = 1):
    """Manifold labels (desc per vertex, asc per tetrahedron), reference ids."""
    W, H, D = dims
    V, E, F, T = counts(dims)
    desc = np.empty(V, np.int32)
    asc = np.empty(T, np.int32)
    bad = lib().orc_labels(W, H, D, np.ascontiguousarray(data, np.float64).reshape(-1), desc, asc, threads)
    if bad:
        raise RuntimeError(f"{bad} label walks hit the step cap")
    return desc, asc


def face_cofaces(faces, dims):
    """(n, 2) cofaces of triangles in get_cell_tetra order, -1 when absent."""
    f = np.ascontiguousarray(faces, np.int32)
    out = np.empty(2 * max(f.size, 1), np.int32)
    lib().orc_face_cofaces(*dims, int(f.size), f if f.size else np.zeros(1, np.int32), out)
    return out[: 2 * f.size].reshape(-1, 2)


def edge_verts(edges, dims):
    """(n, 2) endpoints of edges, higher id first."""
    e = np.ascontiguousarray(edges, np.int32)
    out = np.empty(2 * max(e.size, 1), np.int32)
    lib().orc_edge_verts(*dims, int(e.size), e if e.size else np.zeros(1, np.int32), out)
    return out[: 2 * e.size].reshape(-1, 2)


def mismatch_anchors(P, Q, dims):
    """uint8 per vertex: 1 where a cell anchored there is critical in exactly one pairing."""
    W, H, D = dims
    out = np.zeros(W * H * D, np.uint8)
    lib().orc_mismatch_anchors(W, H, D, *P, *Q, out)
    return out


def link_classes(data, dims):
    """Link components per vertex (lower | upper << 4, uint8) and the counts
    [minima, maxima, regular, join-saddle multiplicity, split-saddle
    multiplicity, sum(1 - chi(lower link))]."""
    W, H, D = dims
    out = np.zeros(W * H * D, np.uint8)
    c = np.zeros(6, np.int64)
    lib().orc_link_classes(W, H, D, np.ascontiguousarray(data, np.float64).reshape(-1), out, c)
    return out, [int(x) for x in c]
