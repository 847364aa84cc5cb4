"""Link-component classification (lower and upper links of every vertex; no
counterpart in the reference, a diagnostic): the oracle against a separate
pure-Python restatement, the Euler characteristic identity, and the minima
against the reference's own unpaired vertices (the fixtures' PV counts)."""
import itertools

import numpy as np
import pytest

from conftest import fixture_files, load_fixture
from oracle import oracle as O

DIRS = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1), (-1, 1, 0), (1, -1, 0), (0, 1, 1),
        (0, -1, -1), (-1, 0, 1), (1, 0, -1), (-1, 1, 1), (1, -1, -1)]
DSET = set(DIRS)


def py_link(data, dims):
    W, H, D = dims
    out = np.zeros(W * H * D, np.uint8)
    counts = [0] * 6
    adj = {(i, j) for i in range(14) for j in range(14)
           if i != j and tuple(a - b for a, b in zip(DIRS[i], DIRS[j])) in DSET}
    for v in range(W * H * D):
        x, y, z = v % W, (v // W) % H, v // (W * H)
        side = {}
        for i, (dx, dy, dz) in enumerate(DIRS):
            nx, ny, nz = x + dx, y + dy, z + dz
            if 0 <= nx < W and 0 <= ny < H and 0 <= nz < D:
                n = nx + ny * W + nz * W * H
                side[i] = -1 if (data[n], n) < (data[v], v) else 1
        comps = []
        for want in (-1, 1):
            nodes = [i for i in side if side[i] == want]
            parent = {i: i for i in nodes}

            def find(a):
                while parent[a] != a:
                    a = parent[a]
                return a
            for a, b in itertools.combinations(nodes, 2):
                if (a, b) in adj:
                    parent[find(a)] = find(b)
            comps.append(len({find(a) for a in nodes}))
        low = [i for i in side if side[i] == -1]
        ne = sum(1 for a, b in itertools.combinations(low, 2) if (a, b) in adj)
        nt = sum(1 for a, b, c in itertools.combinations(low, 3) if (a, b) in adj and (a, c) in adj and (b, c) in adj)
        out[v] = comps[0] | (comps[1] << 4)
        counts[0] += comps[0] == 0
        counts[1] += comps[1] == 0
        counts[2] += comps[0] == 1 and comps[1] == 1
        counts[3] += max(comps[0] - 1, 0)
        counts[4] += max(comps[1] - 1, 0)
        counts[5] += 1 - (len(low) - ne + nt)
    return out, counts


def _fields():
    from dmtz_gb300 import synth

    r = np.random.Generator(np.random.PCG64(5))
    return [("powerlaw", (9, 8, 7), synth.power_law((9, 8, 7), 3).reshape(-1)),
            ("gauss", (7, 6, 9), synth.gaussian_mix((7, 6, 9), 2, n_gauss=6).reshape(-1)),
            ("ties", (6, 7, 5), r.integers(0, 3, size=210).astype(np.float64)),
            ("thin", (12, 2, 3), synth.power_law((12, 2, 3), 1).reshape(-1)),
            ("const", (4, 3, 5), np.full(60, 0.5))]


@pytest.mark.parametrize("name,dims,f", _fields(), ids=[x[0] for x in _fields()])
def test_oracle_matches_python_restatement(name, dims, f):
    got, gc = O.link_classes(f, dims)
    want, wc = py_link(f, dims)
    assert np.array_equal(got, want) and gc == wc
    assert gc[5] == 1  # Euler characteristic of the solid box


@pytest.mark.parametrize("path", fixture_files()[:8], ids=lambda p: p.split("ref_")[-1][:-4])
def test_minima_are_the_reference_unpaired_vertices(path):
    meta, z, f, g = load_fixture(path)
    dims = tuple(meta["dims"])
    out, c = O.link_classes(f, dims)
    assert c[0] == meta["PV_ncrit"] and c[5] == 1
    PV = O.pair(f, dims)[0]
    assert np.array_equal((out & 15) == 0, PV == -1)
