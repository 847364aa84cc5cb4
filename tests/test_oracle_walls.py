"""Wall checks of preserve_connectors = 1 in the oracle (get_false_ds_wall /
fix_ds_wall of main_3d.cu:5064-5121, 5297-5413, restated without the races
of the reference's detection): the C oracle's records against a second,
pure-Python restatement of the same per-2-saddle depth-first search, and
whole corrections that end with no wall record left."""
import numpy as np
import pytest

from oracle import oracle as O


def _case(kind, dims, seed, rel):
    from dmtz_gb300 import synth

    f, g = synth.make_case(kind, dims, seed, rel, "sz" if kind == "powerlaw" else "uniform")
    return f.reshape(-1), g.reshape(-1)


def py_wall_detect(P, Q, dims):
    """Per original 2-saddle face: depth-first search with its own visited set
    over faces reached through original V-paths (face -> edge -> the face the
    edge is paired with); edges (v1 v2), (v1 v3), (v2 v3) of the descending
    vertex triple in that order; the first edge whose original and
    decompressed pairings differ is the record."""
    PV, PE, PF, PT = P
    QE = Q[1]
    F = len(PF)
    tv = O.tri_verts(np.arange(F, dtype=np.int32), dims)
    pairs = np.stack([tv[:, [0, 1]], tv[:, [0, 2]], tv[:, [1, 2]]], axis=1).reshape(-1, 2)
    fe = O.edge_ids(pairs, dims).reshape(F, 3)
    recs = []
    for s in np.flatnonzero(PF == -1):
        visited, stack, rec = set(), [int(s)], None
        while stack and rec is None:
            t = stack.pop()
            if t in visited:
                continue
            visited.add(t)
            for j in fe[t]:
                pe = int(PE[j])
                if pe == -1:
                    continue
                if pe != QE[j]:
                    rec = int(j)
                    break
                if pe != t and 0 <= pe < F and PF[pe] == j:
                    stack.append(pe)
        if rec is not None:
            recs.append((int(s), rec))
    return recs


@pytest.mark.parametrize("kind,dims,seed,rel", [("powerlaw", (12, 11, 10), 1, 1e-2), ("gauss", (14, 12, 10), 2, 1e-2),
                                                ("powerlaw", (9, 13, 11), 4, 1e-3)])
def test_wall_detect_matches_python(kind, dims, seed, rel):
    f, g = _case(kind, dims, seed, rel)
    P, Q = O.pair(f, dims), O.pair(g, dims)
    ws, we, pops, oob = O.wall_detect(P, Q, dims)
    assert oob == 0
    want = py_wall_detect(P, Q, dims)
    assert list(zip(ws.tolist(), we.tolist())) == want
    assert len(want) > 0
    # a gradient agrees with itself: no records, and every search runs to its end
    ws0, _, pops0, _ = O.wall_detect(P, P, dims)
    assert len(ws0) == 0 and pops0 >= pops


@pytest.mark.parametrize("flags", [[1, 1, 1, 0, 1, 0, 0], [1, 1, 0, 0, 1, 0, 0]])
def test_wall_correction_ends_clean(flags):
    dims, rel = (20, 18, 16), 1e-3
    f, g = _case("powerlaw", dims, 1, rel)
    P, Q = O.pair(f, dims), O.pair(g, dims)
    assert len(O.wall_detect(P, Q, dims)[0]) > 0
    out, st, _ = O.correct(f, g, dims, rel, flags, max_outer=300, break_stalls=True)
    assert st["converged"] and st["oob"] == 0
    assert np.all(np.abs(out - f) <= (f.max() - f.min()) * rel * (1 + 1e-12))
    Po = O.pair(out, dims)
    assert len(O.wall_detect(P, Po, dims)[0]) == 0
    assert [len(x) for x in O.cp_mismatch(P, Po, dims)] == [0, 0, 0, 0]
