"""CPU restatement of the warm-start path, for the tests only (the product
path never imports this file).

The reference has no learned part (engine.js starts every run from
f = w_i, src/engine.js:261), so there is nothing of the reference to pin this
against; it restates this project's own definitions so that the CUDA kernels
can be checked:

* ``classes``   - the boundary class of every cell (setupSim's flag rule,
                  src/engine.js:252-254) from the host masks;
* ``features`` / ``targets`` - the R^3 resampling (footprint fractions and
                  means), with an exact Euclidean distance transform where the
                  GPU uses jump flooding;
* ``net_forward`` - the encoder-decoder in torch (CPU, float64), whose
                  autograd gives the reference gradients; with
                  ``bf16_operands`` every convolution rounds its operands to
                  bfloat16 as the tensor-core kernels do (the sums stay
                  float64), so that their gradients can be checked tightly;
* ``apply``     - the warm start: trilinear interpolation of the prediction
                  weighted by voxel fluid fraction and the equilibrium of
                  cpuStep (src/engine.js:288-291).
"""
from __future__ import annotations

import math

import numpy as np

CX = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0])
CY = np.array([0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1])
CZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1])
W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)


def classes(g) -> np.ndarray:
    """0 not fluid, 1 bulk, 2 inlet, 3 outlet, 4 filter, shape (nx, ny, nz)."""
    nx, ny, nz = g.nx, g.ny, g.nz
    fl = g.fluid.reshape(nx, ny, nz).astype(bool)
    op = g.opening.reshape(nx, ny).astype(bool)
    out = g.outlet.reshape(nx, ny, nz).astype(bool)
    dc = g.dc.astype(np.float64)
    filt = (dc > dc[g.top]) & (dc <= g.pleat)
    c = np.where(fl, 1, 0).astype(np.uint8)
    c[fl & filt[None, :, None]] = 4
    c[fl & out] = 3
    inlet = np.zeros_like(fl)
    inlet[:, :, 0] = op & fl[:, :, 0]
    c[inlet] = 2
    return c


def footprint(a: int, n: int, R: int):
    s = n / R
    i0, i1 = math.ceil(a * s - 0.5), math.ceil((a + 1) * s - 0.5)
    if i1 <= i0:
        i0 = min(math.floor((a + 0.5) * s), n - 1)
        i1 = i0 + 1
    return max(i0, 0), min(i1, n)


def _footprints(n, R):
    return [footprint(a, n, R) for a in range(R)]


def _box_sums(arr3: np.ndarray, R: int) -> np.ndarray:
    """Sum of arr3 over every voxel footprint, shape (R, R, R) (int64 / float64)."""
    nx, ny, nz = arr3.shape
    fx, fy, fz = _footprints(nx, R), _footprints(ny, R), _footprints(nz, R)
    sx = np.stack([arr3[a:b].sum(0) for a, b in fx])                       # (R, ny, nz)
    sy = np.stack([sx[:, a:b].sum(1) for a, b in fy], 1)                   # (R, R, nz)
    return np.stack([sy[:, :, a:b].sum(2) for a, b in fz], 2)              # (R, R, R)


def _counts(nx, ny, nz, R):
    lx = np.array([b - a for a, b in _footprints(nx, R)])
    ly = np.array([b - a for a, b in _footprints(ny, R)])
    lz = np.array([b - a for a, b in _footprints(nz, R)])
    return lx[:, None, None] * ly[None, :, None] * lz[None, None, :]


def edt(solid: np.ndarray, sx: float, sy: float, sz: float) -> np.ndarray:
    """Exact distance (scaled axes) from every voxel to the nearest solid voxel (brute force)."""
    R = solid.shape[0]
    pts = np.argwhere(solid).astype(np.float64) * [sx, sy, sz]
    grid = np.stack(np.meshgrid(*(np.arange(R),) * 3, indexing="ij"), -1).reshape(-1, 3) * [sx, sy, sz]
    if len(pts) == 0:
        return np.full((R, R, R), np.inf)
    best = np.full(len(grid), np.inf)
    for i in range(0, len(pts), 256):
        d = ((grid[:, None, :] - pts[None, i:i + 256, :]) ** 2).sum(-1).min(1)
        best = np.minimum(best, d)
    return np.sqrt(best).reshape(R, R, R)


def features(cls: np.ndarray, R: int, K: float, coords: bool = False):
    """Network input (9 or 12, R, R, R) float32 and the exact wall distance (R, R, R) before scaling."""
    nx, ny, nz = cls.shape
    n = _counts(nx, ny, nz, R)
    inv = np.float32(1.0) / n.astype(np.float32)
    cnt = [_box_sums((cls > 0).astype(np.int64), R), _box_sums((cls == 2).astype(np.int64), R),
           _box_sums((cls == 3).astype(np.int64), R), _box_sums((cls == 4).astype(np.int64), R)]
    x = np.zeros((9, R, R, R), np.float32)
    for c in range(4):
        x[c] = cnt[c].astype(np.float32) * inv
    solid = cnt[0] * 2 < n
    d = edt(solid, nx / R, ny / R, nz / R)
    x[4] = np.minimum(d / 20.0, 2.0).astype(np.float32)
    x[5] = np.float32(K) / np.float32(3.0)
    x[6], x[7], x[8] = np.float32(nx) / 128, np.float32(ny) / 64, np.float32(nz) / 128
    if coords:
        c = (np.arange(R, dtype=np.float32) + np.float32(0.5)) / np.float32(R)
        xc = np.zeros((3, R, R, R), np.float32)
        xc[0] = c[:, None, None]
        xc[1] = c[None, :, None]
        xc[2] = c[None, None, :]
        x = np.concatenate([x, xc])
    return x, d


def targets(cls: np.ndarray, avg: dict, R: int, u0: float):
    """Target (4, R, R, R) and weight (R, R, R) from time-averaged fields avg['ux'|'uy'|'uz'|'rho']
    given on the full (nx, ny, nz) grid (zero outside the fluid)."""
    nx, ny, nz = cls.shape
    fl = (cls > 0).astype(np.int64)
    nf = _box_sums(fl, R)
    n = _counts(nx, ny, nz, R)
    t = np.zeros((4, R, R, R))
    with np.errstate(invalid="ignore", divide="ignore"):
        for c, k in enumerate(("ux", "uy", "uz", "rho")):
            t[c] = _box_sums(np.where(fl > 0, avg[k], 0.0).astype(np.float64), R) / nf
    t[:3] /= u0
    t[3] = (t[3] - 1.0) / (5 * u0 * u0)
    t[:, nf == 0] = 0
    return t, nf / n


def conv_layers(base: int, levels: int, n_in: int = 9):
    """(cin, cout, stride, relu) of every convolution, in parameter order."""
    ch = [base << l for l in range(levels)]
    out, c = [], n_in
    for l in range(levels):
        out += [(c, ch[l], 1 if l == 0 else 2, True), (ch[l], ch[l], 1, True)]
        c = ch[l]
    for l in range(levels - 2, -1, -1):
        out += [(ch[l + 1], ch[l], 1, True), (ch[l], ch[l], 1, True)]
    out.append((ch[0], 4, 1, False))
    return out


def unpack(weights: np.ndarray, base: int, levels: int, torch, n_in: int = 9):
    """Per-layer (weight, bias) torch tensors (float64) from the flat parameter vector."""
    off, out = 0, []
    for cin, cout, s, relu in conv_layers(base, levels, n_in):
        nw = cout * cin * 27
        w = torch.tensor(weights[off:off + nw].reshape(cout, cin, 3, 3, 3), dtype=torch.float64, requires_grad=True)
        b = torch.tensor(weights[off + nw:off + nw + cout], dtype=torch.float64, requires_grad=True)
        off += nw + cout
        out.append((w, b, s, relu))
    assert off == weights.size
    return out


def _bf16_conv(torch):
    """A 3x3x3 convolution (padding 1) that rounds its operands to bfloat16
    the way the tensor-core path does: the forward rounds x and w; the data
    gradient rounds the (ReLU-masked) output gradient and w; the weight
    gradient rounds the output gradient and x where that path computes it on
    the tensor cores (output rows of 16, 32 or a multiple of 64 voxels, or
    narrower rows in output planes of a multiple of 64 voxels) and keeps
    float32 operands elsewhere; the bias gradient sums the unrounded output
    gradient."""
    F = torch.nn.functional
    G = torch.nn.grad

    def r(t):
        return t.to(torch.float32).to(torch.bfloat16).to(t.dtype)

    class Bf16Conv(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x, w, b, s):
            xr, wr = r(x), r(w)
            ctx.save_for_backward(x, xr, w, wr)
            ctx.s = s
            return F.conv3d(xr, wr, b, stride=s, padding=1)

        @staticmethod
        def backward(ctx, dy):
            x, xr, w, wr = ctx.saved_tensors
            s, dyr = ctx.s, r(dy)
            dx = G.conv3d_input(x.shape, wr, dyr, stride=s, padding=1)
            wo, ho = dy.shape[-1], dy.shape[-2]
            bw = min(wo, 64)
            tc = (bw in (16, 32, 64) and wo % bw == 0) or (wo < 16 and (ho * wo) % 64 == 0)
            dw = G.conv3d_weight(xr if tc else x, w.shape, dyr if tc else dy, stride=s, padding=1)
            return dx, dw, dy.sum(dim=(0, 2, 3, 4)), None

    return Bf16Conv.apply


def net_forward(layers, x, levels: int, torch, bf16_operands: bool = False):
    """The encoder-decoder of the warm start (x: (B, 9 or 12, R, R, R) float64)."""
    F = torch.nn.functional
    it = iter(layers)
    conv3d = _bf16_conv(torch) if bf16_operands else None

    def conv(t):
        w, b, s, relu = next(it)
        y = conv3d(t, w, b, s) if bf16_operands else F.conv3d(t, w, b, stride=s, padding=1)
        return F.relu(y) if relu else y

    skips, t = [], x
    for l in range(levels):
        t = conv(conv(t))
        skips.append(t)
    for l in range(levels - 2, -1, -1):
        u = F.interpolate(t, scale_factor=2, mode="nearest")
        t = conv(conv(u) + skips[l])
    return conv(t)


def apply(pred: np.ndarray, fluid: np.ndarray, ijk: np.ndarray, grid, u0: float) -> np.ndarray:
    """Warm-start populations f[q, a] (float64) of the fluid cells at ijk (NF, 3)."""
    R = pred.shape[1]
    nx, ny, nz = grid
    f = [(ijk[:, a].astype(np.float32) + np.float32(0.5)) * np.float32(R) / np.float32(n) - np.float32(0.5)
         for a, n in enumerate((nx, ny, nz))]
    lo = [np.clip(np.floor(v).astype(np.int64), 0, R - 2) for v in f]
    wt = [np.clip(v - l, 0.0, 1.0) for v, l in zip(f, lo)]
    acc = np.zeros((4, len(ijk)))
    wsum = np.zeros(len(ijk))
    for corner in range(8):
        d = [(corner >> 2) & 1, (corner >> 1) & 1, corner & 1]
        idx = tuple(lo[a] + d[a] for a in range(3))
        w = np.ones(len(ijk))
        for a in range(3):
            w = w * (wt[a] if d[a] else 1 - wt[a])
        w = w * fluid[idx]
        wsum += w
        acc += w * pred[(slice(None),) + idx]
    p = acc / np.where(wsum > 1e-6, wsum, 1.0)
    near = tuple(np.clip(np.rint(v).astype(np.int64), 0, R - 1) for v in f)
    p = np.where(wsum > 1e-6, p, pred[(slice(None),) + near])
    ux, uy, uz = p[0] * u0, p[1] * u0, p[2] * u0
    rho = np.clip(1 + 5 * u0 * u0 * p[3], 0.9, 1.1)
    sp = np.sqrt(ux * ux + uy * uy + uz * uz)
    r = np.where(sp > 0.2, 0.2 / np.maximum(sp, 1e-300), 1.0)
    ux, uy, uz = ux * r, uy * r, uz * r
    u2 = ux * ux + uy * uy + uz * uz
    out = np.empty((19, len(ijk)))
    for q in range(19):
        cu = CX[q] * ux + CY[q] * uy + CZ[q] * uz
        out[q] = W[q] * rho * (1 + 3 * cu + 4.5 * cu * cu - 1.5 * u2)
    return out
