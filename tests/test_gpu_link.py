"""Link-component classification on the GPU (dmtz_link_classes) against the
oracle, bit for bit per vertex, on the reference-pinned fixtures and the
edge-case grids, and its invariants on the 256^3 benchmark field: the Euler
characteristic identity and minima = the vertices the gradient leaves
unpaired."""
import numpy as np
import pytest

from conftest import fixture_files, load_fixture
from oracle import oracle as O
from test_oracle_link import _fields

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", fixture_files(), ids=lambda p: p.split("ref_")[-1][:-4])
def test_link_classes_match_oracle(gpu_ctx, path):
    meta, z, f, g = load_fixture(path)
    dims = tuple(meta["dims"])
    for data in (f, g):
        got, gc = gpu_ctx.link_classes(data, dims)
        want, wc = O.link_classes(data, dims)
        assert np.array_equal(got, want) and gc == wc
    assert gc[5] == 1


@pytest.mark.parametrize("name,dims,f", _fields(), ids=[x[0] for x in _fields()])
def test_link_classes_edge_cases(gpu_ctx, name, dims, f):
    got, gc = gpu_ctx.link_classes(f, dims)
    want, wc = O.link_classes(f, dims)
    assert np.array_equal(got, want) and gc == wc


def test_link_counts_256(gpu_ctx):
    torch = pytest.importorskip("torch")
    import bench

    f, g = bench.workload(0)
    dims = (256, 256, 256)
    fd = torch.from_numpy(f).cuda()
    c = gpu_ctx.link_counts_ptr(fd.data_ptr(), dims)
    assert c[5] == 1
    PV = gpu_ctx.extract(f, dims)[0]
    assert c[0] == int((PV == -1).sum())
    assert c[0] + c[1] + c[2] <= f.size and c[3] > 0 and c[4] > 0
