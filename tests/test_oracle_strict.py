"""Strict descending separatrix checks in the oracle (no counterpart in the
reference).  The reference's get_false_ds_vpath compares each 1-saddle
endpoint's pairing at the first vertex of its path only, so a corrected field
can keep a descending separatrix that ends at another minimum.  The strict
check walks the whole original path.  On the reference-pinned full-MSC cases,
the strict loop must end with every separatrix label equal to the original's:
the descending label (minimum reached) of both endpoints of every original
1-saddle and the ascending label (maximum reached) of both cofaces of every
original 2-saddle, with no critical cell differing.  The default check must
stay the reference's (its outputs are pinned elsewhere)."""
import numpy as np
import pytest

from conftest import fixture_files, load_fixture
from oracle import oracle as O

SMALL = [p for p in fixture_files() if any(k in p for k in ("g16_1110", "g32_1110000", "t161210", "p201822_1110000"))]


def separatrix_agreement(f, out, dims):
    """(endpoints compared, equal descending labels, cofaces compared, equal
    ascending labels, critical cells differing) from the oracle's labels."""
    P, Q = O.pair(f, dims), O.pair(out, dims)
    dP, aP = O.labels(f, dims)
    dQ, aQ = O.labels(out, dims)
    ev = O.edge_verts(np.nonzero(P[1] == -1)[0].astype(np.int32), dims).reshape(-1)
    cof = O.face_cofaces(np.nonzero(P[2] == -1)[0].astype(np.int32), dims).reshape(-1)
    cof = cof[cof >= 0]
    crit = sum(len(x) for x in O.cp_mismatch(P, Q, dims))
    return len(ev), int((dP[ev] == dQ[ev]).sum()), len(cof), int((aP[cof] == aQ[cof]).sum()), crit


@pytest.mark.parametrize("path", SMALL, ids=lambda p: p.split("ref_")[-1][:-4])
def test_strict_labels_exact(path):
    meta, z, f, g = load_fixture(path)
    dims = tuple(meta["dims"])
    out, st, _ = O.correct(f, g, dims, meta["rel"], meta["flags"], max_outer=500, strict=True, threads=4)
    assert st["converged"] and st["oob"] == 0
    bound = (f.max() - f.min()) * meta["rel"]
    assert np.all(np.abs(out - f) <= bound * (1 + 1e-12))
    nd, de, na, ae, crit = separatrix_agreement(f, out, dims)
    assert crit == 0 and de == nd and ae == na
    # no descending record is left either
    at, ac, d_e, d_v, oob = O.path_detect(O.pair(f, dims), O.pair(out, dims), dims, strict=True)
    assert len(at) == 0 and len(d_e) == 0 and oob == 0


def test_strict_walk_extends_reference_check():
    """Every record of the reference's first-vertex check is also a strict
    record (the first vertex is where the whole-path walk starts), and on the
    uncorrected field the strict check finds at least as many 1-saddles."""
    path = [p for p in SMALL if "g32_1110000" in p][0]
    meta, z, f, g = load_fixture(path)
    dims = tuple(meta["dims"])
    P, Q = O.pair(f, dims), O.pair(g, dims)
    _, _, e0, v0, _ = O.path_detect(P, Q, dims)
    _, _, e1, v1, _ = O.path_detect(P, Q, dims, strict=True)
    ref = dict(zip(e0.tolist(), v0.tolist()))
    strict = dict(zip(e1.tolist(), v1.tolist()))
    assert set(ref) <= set(strict) and len(strict) >= len(ref)
    # a 1-saddle the reference flags at its first endpoint is flagged at the
    # same vertex by the strict walk
    for e, v in ref.items():
        a, b = O.edge_verts(np.array([e], np.int32), dims)[0]
        if v == a:
            assert strict[e] == v
