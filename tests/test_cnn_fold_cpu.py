"""The algebra of the folded-tap convolution (tensor path 2), in float64 on the
CPU: for each (dy, dz) offset one product of the rows shifted by (-1, dy, dz)
with the three x-taps' weights side by side, then

    out[x] = D[x][tap 0] + D[x + 1][tap 1] + D[x + 2][tap 2],

equals the direct 27-tap convolution; with the weight blocks mirrored
(tap 26 - k) it equals the transposed (FLIP) convolution.  The weight block of
x-tap t at offset index u = (dy + 1) + 3 (dz + 1) is tap t + 3u, as the kernel
lays it out."""
import numpy as np


def _conv_direct(x, w, flip):
    """x: (D, H, W, CIN) zero-padded outside; w: (27, COUT, CIN).
    Forward: out[v] = sum_k x[v + d(k)] w[k]; FLIP: out[v] = sum_k x[v - d(k)] w[k]."""
    D, H, W, _ = x.shape
    xp = np.pad(x, ((1, 1), (1, 1), (1, 1), (0, 0)))
    out = np.zeros((D, H, W, w.shape[1]))
    for k in range(27):
        dx, dy, dz = k % 3 - 1, (k // 3) % 3 - 1, k // 9 - 1
        if flip:
            dx, dy, dz = -dx, -dy, -dz
        out += np.einsum("zyxc,nc->zyxn", xp[1 + dz:1 + dz + D, 1 + dy:1 + dy + H, 1 + dx:1 + dx + W], w[k])
    return out


def _conv_folded(x, w, flip):
    """The kernel's scheme: per (dy, dz), rows shifted by (-1, dy, dz) times
    [W(t=0); W(t=1); W(t=2)], then the three column blocks summed with shifts
    of 0, 1, 2 rows along x."""
    D, H, W, _ = x.shape
    cout = w.shape[1]
    xp = np.pad(x, ((1, 1), (1, 1), (1, 3), (0, 0)))  # two more zero columns on +x: rows x + 1, x + 2
    out = np.zeros((D, H, W, cout))
    for u in range(9):
        dy, dz = u % 3 - 1, u // 3 - 1
        taps = [26 - (t + 3 * u) if flip else t + 3 * u for t in range(3)]
        wb = np.concatenate([w[k] for k in taps], axis=0)  # (3 COUT, CIN): the B operand
        rows = xp[1 + dz:1 + dz + D, 1 + dy:1 + dy + H, 0:W + 2]  # x - 1 .. x + W, the A rows
        d = np.einsum("zyxc,nc->zyxn", rows, wb)  # D[x][3 COUT] for x = 0 .. W + 1
        out += d[:, :, 0:W, 0:cout] + d[:, :, 1:W + 1, cout:2 * cout] + d[:, :, 2:W + 2, 2 * cout:]
    return out


def test_folded_taps_equal_direct_convolution():
    rng = np.random.default_rng(3)
    for dims, cin, cout in (((5, 6, 7), 16, 32), ((3, 4, 9), 32, 16), ((4, 3, 2), 32, 32)):
        D, H, W = dims
        x = rng.standard_normal((D, H, W, cin))
        w = rng.standard_normal((27, cout, cin))
        for flip in (False, True):
            want = _conv_direct(x, w, flip)
            got = _conv_folded(x, w, flip)
            assert np.allclose(got, want, rtol=1e-12, atol=1e-10), (dims, flip, np.abs(got - want).max())
