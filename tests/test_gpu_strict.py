"""Strict descending separatrix checks on the GPU (dmtz_opts.strict_separatrices,
dmtz_path_detect_strict) and the separatrix agreement measurement
(dmtz_separatrix_agreement).

The default loop reproduces the reference, whose descending check looks at the
first vertex of each 1-saddle endpoint's path only; the corrected field then
keeps most, not all, descending separatrix labels.  With the strict check the
loop must end with every separatrix label of the original: the records equal
the oracle's strict records, the corrected field equals the oracle's strict
loop bit for bit (host and graph loops), and the labels agree exactly on every
reference-pinned full-MSC case and on the 256^3 benchmark field."""
import numpy as np
import pytest

from conftest import fixture_files, load_fixture
from oracle import oracle as O
from test_oracle_strict import separatrix_agreement

pytestmark = pytest.mark.gpu
FULL_MSC = [p for p in fixture_files() if "_111" in p]


def _id(p):
    return p.split("ref_")[-1][:-4]


@pytest.mark.parametrize("path", fixture_files(), ids=_id)
def test_strict_detect_matches_oracle(gpu_ctx, path):
    meta, z, f, g = load_fixture(path)
    dims = tuple(meta["dims"])
    got = gpu_ctx.path_detect(f, g, dims, strict=True)
    a_t, a_c, d_e, d_v, oob = O.path_detect(O.pair(f, dims, 4), O.pair(g, dims, 4), dims, strict=True)
    assert oob == 0
    assert sorted(zip(got[0].tolist(), got[1].tolist())) == sorted(zip(a_t.tolist(), a_c.tolist()))
    assert sorted(zip(got[2].tolist(), got[3].tolist())) == sorted(zip(d_e.tolist(), d_v.tolist()))


@pytest.mark.parametrize("use_graph", [0, 1], ids=["host_loop", "graph_loop"])
@pytest.mark.parametrize("path", FULL_MSC, ids=_id)
def test_strict_correction_labels_exact(gpu_ctx, path, use_graph):
    meta, z, f, g = load_fixture(path)
    dims = tuple(meta["dims"])
    out, rep, cnt = gpu_ctx.correct(f, g, meta["rel"], meta["flags"], dims=dims, use_graph=use_graph,
                                    return_counter=True, strict=True)
    want, st, wcnt = O.correct(f, g, dims, meta["rel"], meta["flags"], max_outer=500, strict=True,
                               break_stalls=True, threads=4)
    assert rep["converged"] and st["converged"]
    assert np.array_equal(out, want) and np.array_equal(cnt, wcnt)
    assert rep["outer_iterations"] == st["outer_iterations"]
    bound = (f.max() - f.min()) * meta["rel"]
    assert np.all(np.abs(out - f) <= bound * (1 + 1e-12))
    a = gpu_ctx.separatrix_agreement(f, out, dims)
    assert a["crit_differ"] == 0
    assert a["desc_equal"] == a["desc_compared"] > 0
    assert a["asc_equal"] == a["asc_compared"] > 0


@pytest.mark.parametrize("path", [p for p in FULL_MSC if any(k in p for k in ("g32_", "p201822", "t161210"))],
                         ids=_id)
def test_agreement_matches_oracle_labels(gpu_ctx, path):
    """dmtz_separatrix_agreement counts what the oracle's labels give, on the
    default (reference) correction, where descending labels can differ."""
    meta, z, f, g = load_fixture(path)
    dims = tuple(meta["dims"])
    out, rep = gpu_ctx.correct(f, g, meta["rel"], meta["flags"], dims=dims)
    a = gpu_ctx.separatrix_agreement(f, out, dims)
    nd, de, na, ae, crit = separatrix_agreement(f, out, dims)
    assert (a["desc_compared"], a["desc_equal"], a["asc_compared"], a["asc_equal"], a["crit_differ"]) == \
        (nd, de, na, ae, crit)
    # and on the uncorrected field, where much differs
    a0 = gpu_ctx.separatrix_agreement(f, g, dims)
    assert (a0["desc_compared"], a0["desc_equal"], a0["asc_compared"], a0["asc_equal"], a0["crit_differ"]) == \
        separatrix_agreement(f, g, dims)


def test_strict_256_field(gpu_ctx):
    """The 256^3 benchmark field: the strict loop converges within the bound
    with every separatrix label equal; the default loop's output keeps the
    reference's partial descending agreement."""
    torch = pytest.importorskip("torch")
    import bench

    f, g = bench.workload(0)
    dims = (256, 256, 256)
    fd = torch.from_numpy(f).cuda()
    gs = torch.from_numpy(g).cuda()
    gd = gs.clone()
    rep = gpu_ctx.correct_ptr(fd.data_ptr(), gs.data_ptr(), dims, bench.REL_EPS, bench.FLAGS, use_graph=1,
                              strict=True)
    assert rep["converged"]
    bound = float(f.max() - f.min()) * bench.REL_EPS
    assert float((gs - fd).abs().max()) <= bound * (1 + 1e-12)
    a = gpu_ctx.separatrix_agreement(fd.data_ptr(), gs.data_ptr(), dims, on_device=True)
    assert a["crit_differ"] == 0
    assert a["desc_equal"] == a["desc_compared"] > 0 and a["asc_equal"] == a["asc_compared"] > 0
    rep0 = gpu_ctx.correct_ptr(fd.data_ptr(), gd.data_ptr(), dims, bench.REL_EPS, bench.FLAGS, use_graph=1)
    assert rep0["converged"]
    a0 = gpu_ctx.separatrix_agreement(fd.data_ptr(), gd.data_ptr(), dims, on_device=True)
    assert a0["crit_differ"] == 0 and a0["asc_equal"] == a0["asc_compared"]
    assert 0.9 * a0["desc_compared"] < a0["desc_equal"] <= a0["desc_compared"]
