"""Learned proposal on the GPU: the bf16 tensor-core network kernels against
the float64 CPU reference (tests/cnn_ref.py), the feature kernel against the
oracle's pairings, and the learned correction's guarantees checked by the
oracle."""
import numpy as np
import pytest

import cnn_ref as R
from oracle import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def net():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import dmtz_gb300 as dm

    n = dm.Network(0, seed=5)
    yield n
    n.close()


def _params(seed):
    rng = np.random.default_rng(seed)
    p = np.zeros(R.n_params(), np.float32)
    o = 0
    for l, (ci, co) in enumerate(R.LAYERS):
        w = rng.uniform(-1, 1, (27, co, ci)) * np.sqrt(6.0 / (27 * ci))
        if l == 3:
            w[:, 1:, :] = 0.0
            w *= 0.5
        p[o:o + w.size] = w.reshape(-1)
        o += w.size
        b = rng.normal(0, 0.05, co)
        if l == 3:
            b[1:] = 0.0
        p[o:o + co] = b
        o += co
    return p


def _feat(seed, dims):
    W, H, D = dims
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, (D, H, W, 16))
    bits = R.bf16_bits(x)
    return R.from_bf16_bits(bits), torch.from_numpy(bits.reshape(-1, 16).view(np.int16)).cuda().view(torch.bfloat16)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


PATHS = pytest.mark.parametrize("path", [1, 2, 0], ids=["tcgen05", "tcgen05_xfold", "mma_sync"])


@pytest.fixture
def tensor_path(net, path):
    net.set_tensor_path(path)
    yield path
    net.set_tensor_path(2)


@PATHS
@pytest.mark.parametrize("dims", [(8, 8, 4), (13, 11, 9), (21, 6, 5), (40, 35, 3)])
def test_forward_matches_reference(net, tensor_path, dims):
    W, H, D = dims
    p = _params(1)
    net.set_params(p)
    feat_h, feat_d = _feat(2, dims)
    out = torch.empty(W * H * D, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    net.forward(feat_d.data_ptr(), out.data_ptr(), dims)
    got = out.cpu().numpy().reshape(D, H, W).astype(np.float64)
    ref, _ = R.forward(feat_h, p.astype(np.float64))
    assert _rel(got, ref) < 3e-3
    assert np.abs(got - ref).max() < 2e-2 * np.abs(ref).max()
    # the unemulated float64 network is close too (bf16 storage is the only approximation)
    ref64, _ = R.forward(feat_h, p.astype(np.float64), emulate=False)
    assert _rel(got, ref64) < 3e-2


@PATHS
@pytest.mark.parametrize("dims,weighted", [((13, 11, 9), False), ((16, 16, 8), False), ((13, 11, 9), True)])
def test_backward_matches_reference(net, tensor_path, dims, weighted):
    W, H, D = dims
    V = W * H * D
    p = _params(3)
    net.set_params(p)
    feat_h, feat_d = _feat(4, dims)
    rng = np.random.default_rng(5)
    target = rng.uniform(-0.9, 0.9, (D, H, W))
    active = rng.random((D, H, W)) < 0.3
    if weighted:
        active = active * rng.integers(1, 9, (D, H, W))
    out = torch.empty(V, dtype=torch.float32, device="cuda")
    tgt = torch.from_numpy(target.reshape(-1).astype(np.float32)).cuda()
    act = torch.from_numpy(active.reshape(-1).astype(np.uint8)).cuda()
    torch.cuda.synchronize()
    net.forward(feat_d.data_ptr(), out.data_ptr(), dims, train=True)
    loss = net.backward(tgt.data_ptr(), act.data_ptr(), dims)
    grads = net.get_grads().astype(np.float64)
    ref_loss, ref_g = R.loss_and_grad(feat_h, p.astype(np.float64), target, active)
    assert abs(loss - ref_loss) < 2e-3 * ref_loss
    o = 0
    for l, (ci, co) in enumerate(R.LAYERS):
        nw = 27 * ci * co
        gw, rw = grads[o:o + nw], ref_g[o:o + nw]
        gb, rb = grads[o + nw:o + nw + co], ref_g[o + nw:o + nw + co]
        assert _rel(gw, rw) < 2e-2, (l, _rel(gw, rw))
        assert _rel(gb, rb) < 2e-2, (l, _rel(gb, rb))
        if l == 3:
            assert not np.any(gw.reshape(27, co, ci)[:, 1:, :]) and not np.any(gb[1:])
        o += nw + co
    # deterministic: the same pass again gives the same bits
    net.forward(feat_d.data_ptr(), out.data_ptr(), dims, train=True)
    loss2 = net.backward(tgt.data_ptr(), act.data_ptr(), dims)
    assert loss2 == loss
    assert np.array_equal(net.get_grads(), grads.astype(np.float32))


def test_backward_needs_training_forward(net):
    import dmtz_gb300 as dm

    dims = (9, 9, 9)
    V = 729
    _, feat_d = _feat(6, dims)
    out = torch.empty(V, dtype=torch.float32, device="cuda")
    tgt = torch.zeros(V, dtype=torch.float32, device="cuda")
    act = torch.ones(V, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    net.forward(feat_d.data_ptr(), out.data_ptr(), dims, train=False)
    with pytest.raises(dm.DmtzError):
        net.backward(tgt.data_ptr(), act.data_ptr(), dims)
    net.forward(feat_d.data_ptr(), out.data_ptr(), dims, train=True)
    with pytest.raises(dm.DmtzError):
        net.backward(tgt.data_ptr(), act.data_ptr(), (9, 9, 8))


def test_adam_step(net):
    dims = (12, 10, 8)
    V = 960
    p = _params(7)
    net.set_params(p)
    _, feat_d = _feat(8, dims)
    rng = np.random.default_rng(9)
    out = torch.empty(V, dtype=torch.float32, device="cuda")
    tgt = torch.from_numpy(rng.uniform(-0.5, 0.5, V).astype(np.float32)).cuda()
    act = torch.from_numpy((rng.random(V) < 0.5).astype(np.uint8)).cuda()
    torch.cuda.synchronize()
    w = p.astype(np.float64)
    m = np.zeros_like(w)
    v = np.zeros_like(w)
    lr, b1, b2, eps = 1e-3, 0.9, 0.999, 1e-8
    for t in (1, 2):
        net.forward(feat_d.data_ptr(), out.data_ptr(), dims, train=True)
        net.backward(tgt.data_ptr(), act.data_ptr(), dims)
        g = net.get_grads().astype(np.float64)
        net.step(lr)
        m = b1 * m + (1 - b1) * g
        v = b2 * v + (1 - b2) * g * g
        w = w - lr * (m / (1 - b1 ** t)) / (np.sqrt(v / (1 - b2 ** t)) + eps)
        got = net.get_params().astype(np.float64)
        assert np.abs(got - w).max() < 1e-5, t
        w = got  # follow the device's fp32 rounding


def _features_ref(f, g, dims, rel_eps):
    """Channels 0 and 2..15 in float32 numpy; channel 1 and the mask from the oracle."""
    W, H, D = dims
    ff = f.reshape(D, H, W)
    bound = rel_eps * (f.max() - f.min())
    c = np.zeros((D, H, W, 16), np.float64)
    c[..., 0] = np.clip(((g - f) / bound).reshape(D, H, W).astype(np.float32), -1, 1)
    P = O.pair(f, dims)
    Q = O.pair(g, dims)
    mm = O.mismatch_anchors(P, Q, dims).reshape(D, H, W)
    c[..., 1] = mm
    pad = np.pad(ff, 1, constant_values=np.nan)
    dirs = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1), (-1, 1, 0), (1, -1, 0),
            (0, 1, 1), (0, -1, -1), (-1, 0, 1), (1, 0, -1), (-1, 1, 1), (1, -1, -1)]
    for k, (dx, dy, dz) in enumerate(dirs):
        nb = pad[1 + dz:1 + dz + D, 1 + dy:1 + dy + H, 1 + dx:1 + dx + W]
        x = ((nb - ff) / (4.0 * bound)).astype(np.float32)
        c[..., 2 + k] = np.where(np.isnan(nb), 0.0, np.tanh(x))
    act = mm.astype(bool)
    for ax in range(3):
        out = np.zeros_like(act)
        n = act.shape[2 - ax]
        for s in range(-2, 3):
            src = [slice(None)] * 3
            dst = [slice(None)] * 3
            a = 2 - ax
            src[a] = slice(max(s, 0), n + min(s, 0))
            dst[a] = slice(max(-s, 0), n - max(s, 0))
            out[tuple(dst)] |= act[tuple(src)]
        act = out
    return c, act


@pytest.mark.parametrize("dims,seed", [((24, 20, 18), 3), ((33, 17, 9), 11)])
def test_features_match_oracle(gpu_ctx, dims, seed):
    from dmtz_gb300 import synth

    W, H, D = dims
    V = W * H * D
    rel = 1e-3
    f, g = synth.make_case("powerlaw", dims, seed, rel, "sz")
    f, g = f.reshape(-1), g.reshape(-1)
    fd = torch.from_numpy(f).cuda()
    gd = torch.from_numpy(g).cuda()
    feat = torch.empty((V, 16), dtype=torch.bfloat16, device="cuda")
    active = torch.empty(V, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    gpu_ctx.features(fd.data_ptr(), gd.data_ptr(), dims, rel, feat.data_ptr(), active.data_ptr())
    got = R.from_bf16_bits(feat.view(torch.int16).cpu().numpy().view(np.uint16)).reshape(D, H, W, 16)
    ref, ref_act = _features_ref(f, g, dims, rel)
    assert np.array_equal(got[..., 1], ref[..., 1])
    assert got[..., 1].sum() > 0
    assert np.array_equal(active.cpu().numpy().reshape(D, H, W).astype(bool), ref_act)
    # other channels: within one bf16 rounding step of the float32 values
    diff = np.abs(got - R.bf16(ref))
    assert diff.max() <= 2 ** -7 * np.maximum(np.abs(ref), 2 ** -20).max()
    assert (diff > 0).mean() < 0.01


def _oracle_accepts(f, fixed, dims, rel, flags):
    bound = rel * (f.max() - f.min())
    assert np.abs(fixed - f).max() <= bound * (1 + 1e-12)
    P = O.pair(f, dims)
    Q = O.pair(fixed, dims)
    assert all(len(x) == 0 for x in O.cp_mismatch(P, Q, dims))
    if flags[1]:
        at, ac, de, dv, oob = O.path_detect(P, Q, dims)
        assert len(at) == 0 and len(de) == 0


@pytest.mark.parametrize("flags", [(1, 1, 1, 0, 0, 0, 0), (1, 0, 0, 0, 0, 0, 0)])
def test_learned_correction_keeps_guarantees(gpu_ctx, net, flags):
    from dmtz_gb300 import synth

    dims = (40, 36, 32)
    rel = 1e-3
    f, g = synth.make_case("powerlaw", dims, 21, rel, "sz")
    f, g = f.reshape(-1), g.reshape(-1)
    net.set_params(_params(12))
    for use_graph in (0, 1):
        fixed, rep = gpu_ctx.correct_learned(net, f, g, rel, flags, dims=dims, max_rounds=5000, use_graph=use_graph)
        assert rep["converged"], rep
        assert sum(rep["final_mismatch"]) == 0
        assert rep["edited_vertices"] >= int((fixed != g).sum()) > 0
        _oracle_accepts(f, fixed, dims, rel, flags)


def test_training_reduces_loss(gpu_ctx):
    import dmtz_gb300 as dm
    from dmtz_gb300 import learned

    traces = [learned.make_trace(gpu_ctx, *learned.trace_fields((32, 32, 32), 1000 + i, 1e-3), 1e-3)
              for i in range(4)]
    traces = [t for t in traces if t is not None]
    assert traces
    n = dm.Network(0, seed=1)
    hist = learned.train(n, traces, epochs=25, lr=2e-3)
    first = np.mean(hist[:3])
    last = np.mean(hist[-3:])
    assert np.isfinite(hist).all()
    assert last < 0.8 * first, (first, last)
    n.close()


def _proposal(gpu_ctx, net, f, g, dims, rel, min_drop=0.5):
    """The vertices the network's warm start would edit (the rule of
    dmtz_correct_learned: active, and f + bound tanh(o) lowers g by at least
    min_drop x bound), and the active mask."""
    V = f.size
    fd, gd = torch.from_numpy(f).cuda(), torch.from_numpy(g).cuda()
    feat = torch.empty((V, 16), dtype=torch.bfloat16, device="cuda")
    active = torch.empty(V, dtype=torch.uint8, device="cuda")
    out = torch.empty(V, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    gpu_ctx.features(fd.data_ptr(), gd.data_ptr(), dims, rel, feat.data_ptr(), active.data_ptr())
    net.forward(feat.data_ptr(), out.data_ptr(), dims)
    torch.cuda.synchronize()
    bound = rel * float(f.max() - f.min())
    p = fd + bound * torch.tanh(out.double())
    prop = (active > 0) & (gd - p >= min_drop * bound)
    return prop.cpu().numpy(), (active > 0).cpu().numpy()


def test_trained_network_finds_the_loops_edits(gpu_ctx):
    """What training gains: on a held-out field, the vertices the trained
    network proposes to lower are much more often ones the exact loop lowers
    than those of the untrained network, or than active vertices at random.
    (It does not make the loop faster on the benchmark fields: the loop needs
    as many rounds from the proposal, and the network pass costs more than it
    saves; bench.py reports that A/B.)"""
    import dmtz_gb300 as dm
    from dmtz_gb300 import learned

    rel = 1e-4
    traces = [learned.make_trace(gpu_ctx, *learned.trace_fields((64, 64, 64), 3000 + i, rel), rel) for i in range(24)]
    traces = [t for t in traces if t is not None]
    trained = dm.Network(0, seed=0)
    learned.train(trained, traces, epochs=10, lr=1e-3)
    del traces
    untrained = dm.Network(0, seed=0)
    dims = (96, 96, 96)
    f, g = learned.trace_fields(dims, 77, rel)
    f, g = f.reshape(-1), g.reshape(-1)
    fixed, rep = gpu_ctx.correct(f, g, rel, dims=dims, use_graph=1)
    assert rep["converged"]
    edited = fixed < g
    res = {}
    for name, n in (("trained", trained), ("untrained", untrained)):
        prop, active = _proposal(gpu_ctx, n, f, g, dims, rel)
        res[name] = (int(prop.sum()), float((prop & edited).sum() / max(prop.sum(), 1)))
    base = float((edited & active).sum() / active.sum())
    trained.close()
    untrained.close()
    n_tr, prec_tr = res["trained"]
    assert n_tr > 0
    assert prec_tr > 2 * base and prec_tr > res["untrained"][1], (res, base)


def test_tensor_paths_agree(net):
    """tcgen05 and mma.sync convolutions: the same bf16 products and f32 sums,
    only in another order, on a grid of many tiles (128^2 x 24)."""
    dims = (128, 128, 24)
    W, H, D = dims
    net.set_params(_params(9))
    _, feat_d = _feat(10, dims)
    outs = []
    for path in (1, 2, 0):
        net.set_tensor_path(path)
        out = torch.empty(W * H * D, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        net.forward(feat_d.data_ptr(), out.data_ptr(), dims)
        outs.append(out.cpu().numpy().astype(np.float64))
    net.set_tensor_path(2)
    assert _rel(outs[0], outs[2]) < 1e-2
    assert _rel(outs[1], outs[2]) < 1e-2


def test_mma_shape_ceiling(net):
    """The tensor pipe's rate for back-to-back 128 x N x 16 products: every
    shape completes, and wider products run at least as fast per FLOP as the
    convolutions' N = 32 (the rates are the ceilings the profiles cite)."""
    rates = {n: net.mma_ceiling(n, reps=256) for n in (32, 64, 96, 128, 256)}
    assert all(r > 0 for r in rates.values()), rates
    assert rates[256] >= rates[96] >= rates[32], rates
    for bad in (40, 272):  # DmtzError: N is one of 32, 48, 64, 96, 128, 256
        with pytest.raises(RuntimeError):
            net.mma_ceiling(bad)
