"""dmtz_gb300 — GB300 implementation of DMTz's topology-correction path.

Python front end of libdmtz (include/dmtz.h) through ctypes.  The compute
runs in the CUDA library; nothing here falls back to the CPU: every function
raises if the library or a GPU is missing.

    import dmtz_gb300 as dm
    ctx = dm.Context()
    fixed, report = ctx.correct(f, g, rel_eps=1e-4, flags=(1, 1, 1, 0, 0, 0, 0))

Arrays are float64 with shape (D, H, W) or flat, x fastest (the reference's
vertex order).  Pairing arrays use the reference's cell numbering.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

__all__ = ["Context", "DmtzError", "Network", "Opts", "Report", "cell_counts", "load_library"]

_lib = None

STATUS = {0: "OK", 1: "ERR_CUDA", 2: "ERR_ARG", 3: "ERR_IO", 4: "ERR_NONCONVERGED", 5: "ERR_CYCLE",
          6: "ERR_BOUND", 7: "ERR_UNSUPPORTED", 8: "ERR_OOB", 9: "ERR_TOO_LARGE"}


class DmtzError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class Opts(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in (
        "preserve_saddles", "preserve_vpath", "preserve_geometry", "filtration", "preserve_connectors",
        "preserve_type", "edit_type", "max_rounds", "use_graph", "break_stalls", "strict_separatrices")]


class Report(ctypes.Structure):
    _fields_ = [("outer_iterations", ctypes.c_int64), ("cp_rounds", ctypes.c_int64), ("path_rounds", ctypes.c_int64),
                ("initial_mismatch", ctypes.c_int64 * 4), ("final_mismatch", ctypes.c_int64 * 4),
                ("final_paths", ctypes.c_int64 * 2), ("edited_vertices", ctypes.c_int64),
                ("converged", ctypes.c_int32), ("error_flags", ctypes.c_int32), ("seconds", ctypes.c_double),
                ("kernel_launches", ctypes.c_int64), ("phase_ms", ctypes.c_double * 6),
                ("stall_breaks", ctypes.c_int64), ("final_walls", ctypes.c_int64)]

    PHASES = ("pairing", "fix_cp", "path_detect", "fix_path", "apply", "setup")

    def as_dict(self):
        return dict(outer_iterations=self.outer_iterations, cp_rounds=self.cp_rounds, path_rounds=self.path_rounds,
                    initial_mismatch=list(self.initial_mismatch), final_mismatch=list(self.final_mismatch),
                    final_paths=list(self.final_paths), edited_vertices=self.edited_vertices,
                    converged=bool(self.converged),
                    error_flags=self.error_flags, seconds=self.seconds, kernel_launches=self.kernel_launches,
                    stall_breaks=self.stall_breaks, final_walls=self.final_walls,
                    phase_ms=dict(zip(self.PHASES, [round(x, 4) for x in self.phase_ms])))


_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_vp = ctypes.c_void_p
_int = ctypes.c_int


def load_library(build_if_missing: bool = True):
    """Load libdmtz.so (compiling it first if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        _build.build()
    if not os.path.exists(_build.LIB):
        raise OSError(f"libdmtz not built: {_build.LIB}")
    L = ctypes.CDLL(_build.LIB)
    L.dmtz_ctx_create.argtypes = [ctypes.POINTER(_vp), _int]
    L.dmtz_ctx_destroy.argtypes = [_vp]
    L.dmtz_ctx_destroy.restype = None
    L.dmtz_last_error.argtypes = [_vp]
    L.dmtz_last_error.restype = ctypes.c_char_p
    L.dmtz_cell_counts.argtypes = [_int, _int, _int, _i64p]
    L.dmtz_extract.argtypes = [_vp, _int, _int, _int, _vp, _int, _i32p, _i32p, _i32p, _i32p]
    L.dmtz_mismatch.argtypes = [_vp, _int, _int, _int, _f64p, _f64p, _i64p, _i32p, _i32p, _i32p, _i32p]
    L.dmtz_fix_round.argtypes = [_vp, _int, _int, _int, _f64p, _f64p, _i32p, ctypes.c_double, _int, _int, _f64p]
    L.dmtz_path_detect.argtypes = [_vp, _int, _int, _int, _f64p, _f64p, _i64p, _i32p, _i32p, _i32p, _i32p]
    L.dmtz_path_detect_strict.argtypes = [_vp, _int, _int, _int, _f64p, _f64p, _i64p, _i32p, _i32p, _i32p, _i32p]
    L.dmtz_separatrix_agreement.argtypes = [_vp, _int, _int, _int, _vp, _vp, _int, _i64p]
    L.dmtz_link_classes.argtypes = [_vp, _int, _int, _int, _vp, _int, _vp, _i64p]
    L.dmtz_path_detect_connectivity.argtypes = [_vp, _int, _int, _int, _f64p, _f64p, _i64p, _i32p, _i32p, _i32p,
                                                _i32p]
    L.dmtz_path_detect_connectivity.restype = _int
    L.dmtz_wall_detect.argtypes = [_vp, _int, _int, _int, _f64p, _f64p, _i64p, _i32p, _i32p]
    L.dmtz_wall_detect.restype = _int
    L.dmtz_correct.argtypes = [_vp, _int, _int, _int, _vp, _vp, _int, ctypes.c_double, ctypes.POINTER(Opts),
                               ctypes.POINTER(Report), _vp]
    L.dmtz_profile_sweep.argtypes = [_vp, _int, _int, _int, _vp, _vp, _int, _int, _f64p]
    L.dmtz_labels.argtypes = [_vp, _int, _int, _int, _vp, _int, _i32p, _i32p]
    L.dmtz_labels.restype = _int
    L.dmtz_correct_batch.argtypes = [_vp, _int, _vp, ctypes.POINTER(Opts), _vp, _vp, _int]
    L.dmtz_set_tuning.argtypes = [_vp, _int, _int]
    L.dmtz_get_tuning.argtypes = [_vp, ctypes.POINTER(_int), ctypes.POINTER(_int)]
    L.dmtz_autotune.argtypes = [_vp, _int, _int, _int, _vp, _vp, _int, ctypes.POINTER(_int), ctypes.POINTER(ctypes.c_double)]
    L.dmtz_device_name.argtypes = [_vp, ctypes.c_char_p, _int]
    L.dmtz_quantize.argtypes = [_vp, _int, _int, _int, _vp, _vp, _int, ctypes.c_double, ctypes.c_double,
                                ctypes.c_uint64]
    L.dmtz_quantize.restype = _int
    L.dmtz_set_list_reserve.argtypes = [_vp, ctypes.c_double, ctypes.c_int64]
    L.dmtz_set_list_reserve.restype = _int
    # learned proposal
    L.dmtz_cnn_num_params.argtypes = []
    L.dmtz_cnn_num_params.restype = ctypes.c_int64
    L.dmtz_cnn_create.argtypes = [ctypes.POINTER(_vp), _int, ctypes.c_uint64]
    L.dmtz_cnn_destroy.argtypes = [_vp]
    L.dmtz_cnn_destroy.restype = None
    L.dmtz_cnn_last_error.argtypes = [_vp]
    L.dmtz_cnn_last_error.restype = ctypes.c_char_p
    _f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
    L.dmtz_cnn_set_params.argtypes = [_vp, _f32p]
    L.dmtz_cnn_get_params.argtypes = [_vp, _f32p]
    L.dmtz_cnn_get_grads.argtypes = [_vp, _f32p]
    L.dmtz_cnn_forward.argtypes = [_vp, _int, _int, _int, _vp, _vp, _int]
    L.dmtz_cnn_backward.argtypes = [_vp, _int, _int, _int, _vp, _vp, ctypes.POINTER(ctypes.c_double)]
    L.dmtz_cnn_step.argtypes = [_vp, ctypes.c_float]
    L.dmtz_cnn_set_min_drop.argtypes = [_vp, ctypes.c_float]
    L.dmtz_cnn_set_tensor_path.argtypes = [_vp, _int]
    L.dmtz_cnn_mma_ceiling.argtypes = [_vp, _int, _int, ctypes.POINTER(ctypes.c_double)]
    L.dmtz_cnn_set_min_drop.restype = _int
    L.dmtz_cnn_profile.argtypes = [_vp, _int, _int, _int, _vp, _vp, _vp, _vp, _int, _f64p]
    L.dmtz_cnn_profile.restype = _int
    L.dmtz_features.argtypes = [_vp, _int, _int, _int, _vp, _vp, _int, ctypes.c_double, _vp, _vp]
    L.dmtz_correct_learned.argtypes = [_vp, _vp, _int, _int, _int, _vp, _vp, _int, ctypes.c_double,
                                       ctypes.POINTER(Opts), ctypes.POINTER(Report), _vp]
    for fn in ("dmtz_cnn_create", "dmtz_cnn_set_params", "dmtz_cnn_get_params", "dmtz_cnn_get_grads",
               "dmtz_cnn_forward", "dmtz_cnn_backward", "dmtz_cnn_step", "dmtz_features", "dmtz_correct_learned"):
        getattr(L, fn).restype = _int
    for fn in ("dmtz_correct_batch", "dmtz_set_tuning", "dmtz_get_tuning", "dmtz_autotune", "dmtz_device_name"):
        getattr(L, fn).restype = _int
    for fn in ("dmtz_ctx_create", "dmtz_cell_counts", "dmtz_extract", "dmtz_mismatch", "dmtz_fix_round",
               "dmtz_path_detect", "dmtz_correct", "dmtz_profile_sweep"):
        getattr(L, fn).restype = _int
    _lib = L
    return L


def cell_counts(dims):
    W, H, D = dims
    out = np.zeros(4, np.int64)
    rc = load_library().dmtz_cell_counts(W, H, D, out)
    if rc:
        raise DmtzError(rc, "bad dims")
    return tuple(int(x) for x in out)


def _flat(a):
    return np.ascontiguousarray(a, dtype=np.float64).reshape(-1)


def _dims_of(a, dims):
    if dims is not None:
        return tuple(int(x) for x in dims)
    if a.ndim != 3:
        raise ValueError("pass dims=(W, H, D) for flat arrays")
    D, H, W = a.shape
    return (W, H, D)


class Instance(ctypes.Structure):
    """One field of dmtz_correct_batch (see include/dmtz.h)."""
    _fields_ = [("W", ctypes.c_int), ("H", ctypes.c_int), ("D", ctypes.c_int), ("dtype", ctypes.c_int),
                ("orig", ctypes.c_void_p), ("decp", ctypes.c_void_p), ("out", ctypes.c_void_p),
                ("rel_eps", ctypes.c_double)]


class Context:
    """Owns a CUDA device, a stream and the device buffers (dmtz_ctx)."""

    def __init__(self, device: int = 0):
        self._L = load_library()
        h = _vp()
        rc = self._L.dmtz_ctx_create(ctypes.byref(h), device)
        if rc:
            raise DmtzError(rc, "cannot create a context (no CUDA device?)")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.dmtz_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, allow=()):
        if rc and rc not in allow:
            raise DmtzError(rc, self._L.dmtz_last_error(self._h).decode())

    # ------------------------------------------------------------------ stages
    def extract(self, data, dims=None):
        """Gradient pairing of one field -> (PV, PE, PF, PT) in the reference's layout."""
        dims = _dims_of(np.asarray(data), dims)
        d = _flat(data)
        V, E, F, T = cell_counts(dims)
        out = [np.empty(n, np.int32) for n in (V, E, F, T)]
        self._check(self._L.dmtz_extract(self._h, *dims, d.ctypes.data, 0, *out))
        return tuple(out)

    def labels(self, data, dims=None):
        """Manifold labels (descending per vertex, ascending per tetrahedron, reference ids)."""
        dims = _dims_of(np.asarray(data), dims)
        d = _flat(data)
        V, E, F, T = cell_counts(dims)
        desc, asc = np.empty(V, np.int32), np.empty(T, np.int32)
        self._check(self._L.dmtz_labels(self._h, *dims, d.ctypes.data, 0, desc, asc))
        return desc, asc

    def mismatch(self, f, g, dims=None):
        """Sorted critical-cell mismatch lists (min, 1-saddle, 2-saddle, max)."""
        dims = _dims_of(np.asarray(f), dims)
        V, E, F, T = cell_counts(dims)
        c = np.zeros(4, np.int64)
        lists = [np.empty(max(n, 1), np.int32) for n in (V, E, F, T)]
        self._check(self._L.dmtz_mismatch(self._h, *dims, _flat(f), _flat(g), c, *lists))
        return [lists[k][: int(c[k])].copy() for k in range(4)]

    def fix_round(self, f, g, cnt, rel_eps, preserve_saddles, edit_type, dims=None):
        """Delta buffer of one critical-point fix round (sentinel -2000*range where nothing is requested)."""
        dims = _dims_of(np.asarray(f), dims)
        V = cell_counts(dims)[0]
        out = np.empty(V, np.float64)
        self._check(self._L.dmtz_fix_round(self._h, *dims, _flat(f), _flat(g), np.ascontiguousarray(cnt, np.int32),
                                           float(rel_eps), int(preserve_saddles), int(edit_type), out))
        return out

    def wall_detect(self, f, g, dims=None):
        """Wall records of preserve_connectors = 1: (2-saddle faces, first
        differing edges of their walls), sorted by face."""
        dims = _dims_of(np.asarray(f), dims)
        V, E, F, T = cell_counts(dims)
        c = np.zeros(1, np.int64)
        ws, we = np.empty(F, np.int32), np.empty(F, np.int32)
        self._check(self._L.dmtz_wall_detect(self._h, *dims, _flat(f), _flat(g), c, ws, we))
        n = int(c[0])
        return ws[:n].copy(), we[:n].copy()

    def path_detect(self, f, g, dims=None, connectivity=False, strict=False):
        """Separatrix records (as_tet, as_cur, ds_edge, ds_vert), sorted: geometry
        mode, or connectivity mode (ds_vert = trouble maker); strict: whole-path
        descending checks (dmtz_path_detect_strict)."""
        dims = _dims_of(np.asarray(f), dims)
        V, E, F, T = cell_counts(dims)
        c = np.zeros(2, np.int64)
        at, ac = np.empty(F, np.int32), np.empty(F, np.int32)
        de, dv = np.empty(E, np.int32), np.empty(E, np.int32)
        fn = self._L.dmtz_path_detect_connectivity if connectivity else (
            self._L.dmtz_path_detect_strict if strict else self._L.dmtz_path_detect)
        self._check(fn(self._h, *dims, _flat(f), _flat(g), c, at, ac, de, dv))
        na, nd = int(c[0]), int(c[1])
        return at[:na].copy(), ac[:na].copy(), de[:nd].copy(), dv[:nd].copy()

    def correct(self, f, g, rel_eps, flags=(1, 1, 1, 0, 0, 0, 0), dims=None, max_rounds=0, use_graph=0,
                return_counter=False, break_stalls=True, strict=False):
        """Full correction of g against f.  Returns (corrected g, report dict[, edit counter]).
        strict: whole-path descending separatrix checks (dmtz_opts.strict_separatrices)."""
        dims = _dims_of(np.asarray(f), dims)
        ff = _flat(f)
        gg = np.array(_flat(g), copy=True)
        V = ff.size
        cnt = np.empty(V, np.int32)
        o = Opts(*[int(x) for x in flags], int(max_rounds), int(use_graph), int(bool(break_stalls)), int(bool(strict)))
        r = Report()
        rc = self._L.dmtz_correct(self._h, *dims, ff.ctypes.data, gg.ctypes.data, 0, float(rel_eps),
                                  ctypes.byref(o), ctypes.byref(r), cnt.ctypes.data)
        self._check(rc)
        rep = r.as_dict()
        rep["edited_vertices"] = int((gg != _flat(g)).sum())
        return (gg, rep, cnt) if return_counter else (gg, rep)

    def correct_batch(self, fields, flags=(1, 1, 1, 0, 0, 0, 0), workers=8, max_rounds=0, use_graph=1,
                      break_stalls=True):
        """Correct many fields of any sizes in one call.

        fields: iterable of (f, g, rel_eps) with f, g float32 or float64 arrays of
        shape (D, H, W).  Returns a list of (corrected float64 array (D, H, W),
        report dict, status int); status 0 = converged."""
        fields = list(fields)
        keep, insts, outs = [], [], []
        for f, g, rel in fields:
            f = np.ascontiguousarray(f)
            g = np.ascontiguousarray(g, dtype=f.dtype)
            if f.dtype not in (np.float32, np.float64) or f.ndim != 3 or g.shape != f.shape:
                raise ValueError("fields must be float32/float64 arrays of shape (D, H, W)")
            D, H, W = f.shape
            out = np.empty(f.shape, np.float64)
            keep += [f, g]
            outs.append(out)
            insts.append(Instance(W, H, D, 0 if f.dtype == np.float64 else 1, f.ctypes.data, g.ctypes.data,
                                  out.ctypes.data, float(rel)))
        n = len(insts)
        arr = (Instance * max(n, 1))(*insts)
        reps = (Report * max(n, 1))()
        sts = np.zeros(max(n, 1), np.int32)
        o = Opts(*[int(x) for x in flags], int(max_rounds), int(use_graph), int(bool(break_stalls)))
        self._L.dmtz_correct_batch(self._h, n, ctypes.cast(arr, ctypes.c_void_p), ctypes.byref(o),
                                   ctypes.cast(reps, ctypes.c_void_p), sts.ctypes.data, int(workers))
        return [(outs[i], reps[i].as_dict(), int(sts[i])) for i in range(n)]

    def device_name(self):
        buf = ctypes.create_string_buffer(256)
        self._check(self._L.dmtz_device_name(self._h, buf, 256))
        return buf.value.decode()

    def set_tuning(self, shape, blocks_per_sm):
        self._check(self._L.dmtz_set_tuning(self._h, int(shape), int(blocks_per_sm)))

    def quantize(self, f, rel_eps, noise_frac=0.05, seed=0, dims=None):
        """Decompression model on the GPU (host arrays): SZ-style quantisation of
        f with bin 2 eps plus seeded noise on a fraction of the vertices,
        clamped to f +- eps.  Returns g (float64, flat)."""
        dims = _dims_of(np.asarray(f), dims)
        ff = _flat(f)
        gg = np.empty_like(ff)
        self._check(self._L.dmtz_quantize(self._h, *dims, ff.ctypes.data, gg.ctypes.data, 0, float(rel_eps),
                                          float(noise_frac), ctypes.c_uint64(int(seed) & (2**64 - 1))))
        return gg

    def quantize_ptr(self, f_ptr: int, g_ptr: int, dims, rel_eps, noise_frac=0.05, seed=0):
        """quantize on device buffers (float64)."""
        self._check(self._L.dmtz_quantize(self._h, *dims, _vp(f_ptr), _vp(g_ptr), 1, float(rel_eps),
                                          float(noise_frac), ctypes.c_uint64(int(seed) & (2**64 - 1))))

    def set_list_reserve(self, fraction=1.0 / 16, min_entries=1 << 20):
        """Initial room of the mismatch lists (fraction of cells, at least
        min_entries); they grow on demand, results do not depend on it."""
        self._check(self._L.dmtz_set_list_reserve(self._h, float(fraction), int(min_entries)))

    def get_tuning(self):
        a, b = _int(), _int()
        self._check(self._L.dmtz_get_tuning(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def autotune(self, f, g, dims=None):
        """Time the gradient sweep for every brick shape / blocks-per-SM choice on
        (f, g); keep the fastest in this context.  Returns (shape, blocks_per_sm, ms)."""
        dims = _dims_of(np.asarray(f), dims)
        ff, gg = _flat(f), _flat(g)
        best = (_int * 2)()
        ms = ctypes.c_double()
        self._check(self._L.dmtz_autotune(self._h, *dims, ff.ctypes.data, gg.ctypes.data, 0, best, ctypes.byref(ms)))
        return best[0], best[1], ms.value

    def correct_ptr(self, f_ptr: int, g_ptr: int, dims, rel_eps, flags=(1, 1, 1, 0, 0, 0, 0), on_device=True,
                    max_rounds=0, use_graph=0, allow_nonconverged=False, break_stalls=True, strict=False):
        """Correction on raw float64 buffers (device pointers when on_device, else host
        pointers, e.g. pinned memory); g is edited in place.  With
        allow_nonconverged, hitting max_rounds returns the report (converged
        False) instead of raising."""
        o = Opts(*[int(x) for x in flags], int(max_rounds), int(use_graph), int(bool(break_stalls)), int(bool(strict)))
        r = Report()
        self._check(self._L.dmtz_correct(self._h, *dims, _vp(f_ptr), _vp(g_ptr), int(bool(on_device)),
                                         float(rel_eps), ctypes.byref(o), ctypes.byref(r), None),
                    allow=(4,) if allow_nonconverged else ())
        return r.as_dict()

    def separatrix_agreement(self, f, g, dims=None, on_device=False):
        """Labels of g's gradient against f's at the original saddles: dict with
        the 1-saddle endpoints compared / with equal descending labels, the
        2-saddle cofaces compared / with equal ascending labels, and the cells
        whose criticality differs.  f, g: host arrays, or device pointers
        (ints) with on_device and dims."""
        out = np.zeros(5, np.int64)
        if on_device:
            self._check(self._L.dmtz_separatrix_agreement(self._h, *dims, _vp(f), _vp(g), 1, out))
        else:
            dims = _dims_of(np.asarray(f), dims)
            ff, gg = _flat(f), _flat(g)
            self._check(self._L.dmtz_separatrix_agreement(self._h, *dims, ff.ctypes.data, gg.ctypes.data, 0, out))
        return {"desc_compared": int(out[0]), "desc_equal": int(out[1]), "asc_compared": int(out[2]),
                "asc_equal": int(out[3]), "crit_differ": int(out[4])}

    def link_classes(self, data, dims=None, per_vertex=True):
        """Link components per vertex (uint8: lower | upper << 4, or None) and
        the counts [minima, maxima, regular, join-saddle multiplicity,
        split-saddle multiplicity, sum(1 - chi(lower link))]."""
        dims = _dims_of(np.asarray(data), dims)
        d = _flat(data)
        out = np.zeros(d.size, np.uint8) if per_vertex else None
        c = np.zeros(6, np.int64)
        self._check(self._L.dmtz_link_classes(self._h, *dims, d.ctypes.data, 0,
                                              out.ctypes.data if per_vertex else None, c))
        return out, [int(x) for x in c]

    def link_counts_ptr(self, data_ptr: int, dims):
        """The counts of link_classes for a device buffer."""
        c = np.zeros(6, np.int64)
        self._check(self._L.dmtz_link_classes(self._h, *dims, _vp(data_ptr), 1, None, c))
        return [int(x) for x in c]

    def profile_sweep(self, f_ptr: int, g_ptr: int, dims, reps=10, on_device=True):
        """Mean per-launch ms of the six gradient-sweep kernels and of the whole sweep."""
        ms = np.zeros(7, np.float64)
        self._check(self._L.dmtz_profile_sweep(self._h, *dims, _vp(f_ptr), _vp(g_ptr), int(bool(on_device)),
                                               int(reps), ms))
        return ms

    # --------------------------------------------------------- learned proposal
    def features(self, f_ptr: int, g_ptr: int, dims, rel_eps, feat_ptr: int, active_ptr: int, on_device=True):
        """Network input (V x 16 bf16) and active mask (V bytes) of (f, g) into
        device buffers feat_ptr / active_ptr."""
        self._check(self._L.dmtz_features(self._h, *dims, _vp(f_ptr), _vp(g_ptr), int(bool(on_device)),
                                          float(rel_eps), _vp(feat_ptr), _vp(active_ptr)))

    def correct_learned(self, net, f, g, rel_eps, flags=(1, 1, 1, 0, 0, 0, 0), dims=None, max_rounds=0,
                        use_graph=0, break_stalls=True):
        """Correction started from the network's proposal (host arrays).
        Returns (corrected g, report dict)."""
        dims = _dims_of(np.asarray(f), dims)
        ff = _flat(f)
        gg = np.array(_flat(g), copy=True)
        o = Opts(*[int(x) for x in flags], int(max_rounds), int(use_graph), int(bool(break_stalls)))
        r = Report()
        self._check(self._L.dmtz_correct_learned(self._h, net._h, *dims, ff.ctypes.data, gg.ctypes.data, 0,
                                                 float(rel_eps), ctypes.byref(o), ctypes.byref(r), None))
        return gg, r.as_dict()

    def correct_learned_ptr(self, net, f_ptr: int, g_ptr: int, dims, rel_eps, flags=(1, 1, 1, 0, 0, 0, 0),
                            on_device=True, max_rounds=0, use_graph=0, allow_nonconverged=False,
                            break_stalls=True):
        """correct_learned on raw float64 buffers (g edited in place)."""
        o = Opts(*[int(x) for x in flags], int(max_rounds), int(use_graph), int(bool(break_stalls)))
        r = Report()
        self._check(self._L.dmtz_correct_learned(self._h, net._h, *dims, _vp(f_ptr), _vp(g_ptr),
                                                 int(bool(on_device)), float(rel_eps), ctypes.byref(o),
                                                 ctypes.byref(r), None),
                    allow=(4,) if allow_nonconverged else ())
        return r.as_dict()


class Network:
    """The learned-proposal network (dmtz_cnn): 3x3x3 convolutions 16 -> 32 ->
    32 -> 32 -> 1 with bf16 tensor-core kernels.  Buffers passed by pointer are
    device buffers (e.g. torch tensors' data_ptr())."""

    def __init__(self, device: int = 0, seed: int = 0):
        self._L = load_library()
        h = _vp()
        rc = self._L.dmtz_cnn_create(ctypes.byref(h), int(device), ctypes.c_uint64(int(seed) & (2**64 - 1)))
        if rc:
            raise DmtzError(rc, "cannot create the network (no CUDA device?)")
        self._h = h
        self.n_params = int(self._L.dmtz_cnn_num_params())

    def close(self):
        if getattr(self, "_h", None):
            self._L.dmtz_cnn_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc:
            raise DmtzError(rc, self._L.dmtz_cnn_last_error(self._h).decode())

    def get_params(self):
        out = np.empty(self.n_params, np.float32)
        self._check(self._L.dmtz_cnn_get_params(self._h, out))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        if p.size != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters")
        self._check(self._L.dmtz_cnn_set_params(self._h, p))

    def get_grads(self):
        out = np.empty(self.n_params, np.float32)
        self._check(self._L.dmtz_cnn_get_grads(self._h, out))
        return out

    def forward(self, feat_ptr: int, out_ptr: int, dims, train=False):
        self._check(self._L.dmtz_cnn_forward(self._h, *dims, _vp(feat_ptr), _vp(out_ptr), int(bool(train))))

    def backward(self, target_ptr: int, active_ptr: int, dims) -> float:
        loss = ctypes.c_double()
        self._check(self._L.dmtz_cnn_backward(self._h, *dims, _vp(target_ptr), _vp(active_ptr), ctypes.byref(loss)))
        return loss.value

    def set_tensor_path(self, path: int):
        """2: convolutions on tcgen05 with the three x-taps of each offset
        folded into one wider product (default); 1: on tcgen05, one product
        per tap; 0: on mma.sync."""
        self._check(self._L.dmtz_cnn_set_tensor_path(self._h, int(path)))

    def mma_ceiling(self, n: int = 32, reps: int = 512) -> float:
        """TFLOP/s of back-to-back tcgen05.mma of shape 128 x n x 16 (bf16) on
        every SM: the tensor pipe's ceiling for the convolutions' products
        (n = 96 on the default tensor path, 32 on path 1)."""
        t = ctypes.c_double()
        self._check(self._L.dmtz_cnn_mma_ceiling(self._h, int(n), int(reps), ctypes.byref(t)))
        return t.value

    def set_min_drop(self, min_drop: float):
        """Apply the proposal only where it lowers g by at least min_drop x bound."""
        self._check(self._L.dmtz_cnn_set_min_drop(self._h, ctypes.c_float(min_drop)))

    def step(self, lr: float):
        self._check(self._L.dmtz_cnn_step(self._h, ctypes.c_float(lr)))

    def profile(self, feat_ptr: int, out_ptr: int, target_ptr: int, active_ptr: int, dims, reps=5):
        """ms of: forward, training step, one 32->32 conv launch, one 32x32 weight-gradient launch."""
        ms = np.zeros(4, np.float64)
        self._check(self._L.dmtz_cnn_profile(self._h, *dims, _vp(feat_ptr), _vp(out_ptr), _vp(target_ptr),
                                             _vp(active_ptr), int(reps), ms))
        return ms

    def save(self, path):
        np.save(path, self.get_params())

    def load(self, path):
        self.set_params(np.load(path))
