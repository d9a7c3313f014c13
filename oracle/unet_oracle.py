"""CPU oracle of the learned pressure preconditioner (test infrastructure only).

A numpy restatement of the network and of the two-level preconditioner built in
flux-interpolated-advection_gb300/csrc/fia_unet.cu, used by the tests to check the GPU
forward pass, the GPU gradients (backward data and backward weights) and the fine-grid
pieces (restriction, trilinear prolongation, Jacobi term, energy-norm loss).  The reference
program has no learned preconditioner (it solves the projection with amgcl,
calc_pressure_3d.cpp:141-166), so this oracle is pinned by finite differences of its own
loss (tests/test_unet_oracle.py), not by reference outputs.

With rounding=True the oracle rounds to bfloat16 (round to nearest even) at the points where
the GPU stores or stages BF16 values: weights; convolution inputs staged from FP32 sources;
pooled averages; hidden activations after the ReLU; output gradients after the ReLU gate.
Accumulation is in float64 here and FP32 on the GPU.

Layout: tensors are (X, Y, Z, C) arrays (z fastest, channels last); the weights of a layer
are (27, cin, cout) with tap = 9 dx + 3 dy + dz for offsets (dx-1, dy-1, dz-1); the
parameter vector is the layers' weights in order, then omega.
"""
import numpy as np

# (level, cin, cout, relu, mode, in0, in1, out) -- same table as fia_unet.cu kDefs
T_X0, T_A0, T_S0, T_A1, T_S1, T_A2, T_S2, T_A3, T_B3, T_U2, T_C2, T_U1, T_C1, T_U0, T_C0, T_Y = range(16)
PLAIN, POOL, UPCAT, SCALAR = 0, 1, 2, 3
LAYERS = [
    (0, 1, 16, 1, SCALAR, T_X0, -1, T_A0),
    (0, 16, 16, 1, PLAIN, T_A0, -1, T_S0),
    (1, 16, 32, 1, POOL, T_S0, -1, T_A1),
    (1, 32, 32, 1, PLAIN, T_A1, -1, T_S1),
    (2, 32, 48, 1, POOL, T_S1, -1, T_A2),
    (2, 48, 48, 1, PLAIN, T_A2, -1, T_S2),
    (3, 48, 64, 1, POOL, T_S2, -1, T_A3),
    (3, 64, 64, 1, PLAIN, T_A3, -1, T_B3),
    (2, 112, 48, 1, UPCAT, T_B3, T_S2, T_U2),
    (2, 48, 48, 1, PLAIN, T_U2, -1, T_C2),
    (1, 80, 32, 1, UPCAT, T_C2, T_S1, T_U1),
    (1, 32, 32, 1, PLAIN, T_U1, -1, T_C1),
    (0, 48, 16, 1, UPCAT, T_C1, T_S0, T_U0),
    (0, 16, 16, 1, PLAIN, T_U0, -1, T_C0),
    (0, 16, 1, 0, PLAIN, T_C0, -1, T_Y),
]


def num_parameters():
    return sum(27 * l[1] * l[2] for l in LAYERS) + 1


def layer_weights(params, i):
    o = sum(27 * l[1] * l[2] for l in LAYERS[:i])
    cin, cout = LAYERS[i][1], LAYERS[i][2]
    return params[o:o + 27 * cin * cout].reshape(27, cin, cout)


def bf16(a):
    """float32 -> bfloat16 -> float32, round to nearest even."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    b = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def level_dims(fine):
    dims, d = [], [(n + 1) // 2 for n in fine]
    for _ in range(4):
        dims.append(tuple(d))
        d = [(n + 1) // 2 for n in d]
    return dims


def conv(x, W):
    """zero-padded 3x3x3 convolution, x (X,Y,Z,Cin), W (27,Cin,Cout)"""
    X, Y, Z, _ = x.shape
    xp = np.pad(x, ((1, 1), (1, 1), (1, 1), (0, 0)))
    out = np.zeros((X, Y, Z, W.shape[2]))
    for t in range(27):
        dx, dy, dz = t // 9, (t // 3) % 3, t % 3
        out += xp[dx:dx + X, dy:dy + Y, dz:dz + Z, :] @ W[t]
    return out


def conv_backward(x, W, g):
    """gradients of conv(x, W) for output gradient g: (dx, dW)"""
    X, Y, Z, _ = x.shape
    xp = np.pad(x, ((1, 1), (1, 1), (1, 1), (0, 0)))
    dxp = np.zeros_like(xp)
    dW = np.zeros_like(W)
    g2 = g.reshape(-1, g.shape[3])
    for t in range(27):
        dx, dy, dz = t // 9, (t // 3) % 3, t % 3
        xs = xp[dx:dx + X, dy:dy + Y, dz:dz + Z, :]
        dW[t] = xs.reshape(-1, xs.shape[3]).T @ g2
        dxp[dx:dx + X, dy:dy + Y, dz:dz + Z, :] += g @ W[t].T
    return dxp[1:-1, 1:-1, 1:-1, :], dW


def child_counts(fine, coarse):
    cx = np.minimum(2, fine[0] - 2 * np.arange(coarse[0]))
    cy = np.minimum(2, fine[1] - 2 * np.arange(coarse[1]))
    cz = np.minimum(2, fine[2] - 2 * np.arange(coarse[2]))
    cnt = cx[:, None, None] * cy[None, :, None] * cz[None, None, :]
    return cnt


def pool(x, coarse):
    """mean of the (existing) 2x2x2 children"""
    fine = x.shape[:3]
    out = np.zeros(tuple(coarse) + x.shape[3:])
    for i in range(2):
        for j in range(2):
            for k in range(2):
                sub = x[i::2, j::2, k::2]
                out[:sub.shape[0], :sub.shape[1], :sub.shape[2]] += sub
    cnt = child_counts(fine, coarse)
    return out / cnt.reshape(cnt.shape + (1,) * (x.ndim - 3))


def pool_adjoint(g, fine):
    coarse = g.shape[:3]
    cnt = child_counts(fine, coarse)
    gc = g / cnt.reshape(cnt.shape + (1,) * (g.ndim - 3))
    out = np.zeros(tuple(fine) + g.shape[3:])
    for i in range(2):
        for j in range(2):
            for k in range(2):
                sub = out[i::2, j::2, k::2]
                sub += gc[:sub.shape[0], :sub.shape[1], :sub.shape[2]]
    return out


def up(x, fine):
    ix = np.arange(fine[0]) // 2
    iy = np.arange(fine[1]) // 2
    iz = np.arange(fine[2]) // 2
    return x[ix][:, iy][:, :, iz]


def up_adjoint(g, coarse):
    out = np.zeros(tuple(coarse) + g.shape[3:])
    for i in range(2):
        for j in range(2):
            for k in range(2):
                sub = g[i::2, j::2, k::2]
                out[:sub.shape[0], :sub.shape[1], :sub.shape[2]] += sub
    return out


class UNet:
    """forward / backward of the network on a level-0 scalar input x0 (shape dims[0])."""

    def __init__(self, params, fine, rounding=True):
        self.p = np.asarray(params, dtype=np.float64)
        self.dims = level_dims(fine)
        self.r = rounding

    def _rd(self, a):
        return bf16(a) if self.r else a

    def _input(self, i, act):
        lev, cin, cout, relu, mode, in0, in1, out = LAYERS[i]
        if mode == SCALAR:
            return self._rd(act[in0][..., None])
        if mode == PLAIN:
            return act[in0]
        if mode == POOL:
            return self._rd(pool(act[in0], self.dims[lev]))
        return np.concatenate([up(act[in0], self.dims[lev]), act[in1]], axis=3)

    def forward(self, x0):
        act = {T_X0: np.asarray(x0, dtype=np.float64).reshape(self.dims[0])}
        for i, (lev, cin, cout, relu, mode, in0, in1, out) in enumerate(LAYERS):
            W = self._rd(layer_weights(self.p, i))
            y = conv(self._input(i, act), W)
            if relu:
                y = self._rd(np.maximum(y, 0.0))
            act[out] = y if out != T_Y else y[..., 0]
        self.act = act
        return act[T_Y]

    def backward(self, gy):
        """parameter gradient (omega entry 0) for dL/dy = gy, after forward()"""
        act = self.act
        grads = {T_Y: np.asarray(gy, dtype=np.float64).reshape(self.dims[0])[..., None]}
        for t in (T_S0, T_S1, T_S2):
            grads[t] = np.zeros_like(act[t])
        gp = np.zeros(num_parameters())
        for i in reversed(range(len(LAYERS))):
            lev, cin, cout, relu, mode, in0, in1, out = LAYERS[i]
            g = grads[out]
            if relu:
                g = g * (act[out] > 0)
            g = self._rd(g)
            x = self._input(i, act)
            W = self._rd(layer_weights(self.p, i))
            dx, dW = conv_backward(x, W, g)
            o = sum(27 * l[1] * l[2] for l in LAYERS[:i])
            gp[o:o + dW.size] = dW.ravel()
            if i == 0:
                break
            if mode == PLAIN:
                grads[in0] = dx
            elif mode == POOL:
                grads[in0] = grads[in0] + pool_adjoint(dx, self.dims[lev - 1])
            else:
                cu = act[in0].shape[3]
                grads[in0] = up_adjoint(dx[..., :cu], self.dims[lev + 1])
                grads[in1] = grads[in1] + dx[..., cu:]
        return gp


# ---------------------------------------------------------------------------------
# fine-grid pieces: B = -A (7-point, walls and solids Neumann, pinned cell Dirichlet)
# ---------------------------------------------------------------------------------
def excluded_mask(fine, pin, solid=None):
    ex = np.zeros(fine, dtype=bool) if solid is None else solid.reshape(fine).astype(bool).copy()
    ex.reshape(-1)[pin] = True
    return ex


def diag_B(fine, solid=None):
    """number of non-solid neighbours of each cell"""
    s = np.zeros(fine, dtype=bool) if solid is None else solid.reshape(fine).astype(bool)
    d = np.zeros(fine)
    for ax in range(3):
        for sh in (1, -1):
            nb = np.roll(~s, sh, axis=ax).astype(float)
            idx = [slice(None)] * 3
            idx[ax] = 0 if sh == 1 else -1
            nb[tuple(idx)] = 0.0
            d += nb
    return d


def apply_B(x, fine, pin, solid=None):
    """B x on the free cells (0 on excluded cells); x is 0 on the pinned cell"""
    x = np.asarray(x, dtype=np.float64).reshape(fine)
    ex = excluded_mask(fine, pin, solid)
    s = np.zeros(fine, dtype=bool) if solid is None else solid.reshape(fine).astype(bool)
    xv = np.where(ex, 0.0, x)
    out = diag_B(fine, solid) * xv
    for ax in range(3):
        for sh in (1, -1):
            nb = np.roll(xv, sh, axis=ax)
            idx = [slice(None)] * 3
            idx[ax] = 0 if sh == 1 else -1
            nb[tuple(idx)] = 0.0
            out -= nb
    out[ex] = 0.0
    return out


def restrict(r, fine, coarse):
    return pool(np.asarray(r, dtype=np.float64).reshape(fine), coarse)


def _pro_axis(nf, nc):
    """(nf x nc) cell-centred linear prolongation matrix along one axis, clamped"""
    P = np.zeros((nf, nc))
    for i in range(nf):
        if i % 2:
            j0, j1, w0, w1 = i // 2, i // 2 + 1, 0.75, 0.25
        else:
            j0, j1, w0, w1 = i // 2 - 1, i // 2, 0.25, 0.75
        P[i, min(max(j0, 0), nc - 1)] += w0
        P[i, min(max(j1, 0), nc - 1)] += w1
    return P


def prolong(y, fine):
    y = np.asarray(y, dtype=np.float64)
    Px, Py, Pz = (_pro_axis(fine[a], y.shape[a]) for a in range(3))
    return np.einsum("ia,jb,kc,abc->ijk", Px, Py, Pz, y)


def prolong_adjoint(g, coarse):
    g = np.asarray(g, dtype=np.float64)
    Px, Py, Pz = (_pro_axis(g.shape[a], coarse[a]) for a in range(3))
    return np.einsum("ia,jb,kc,ijk->abc", Px, Py, Pz, g)


def precondition(params, r, fine, pin, solid=None, rounding=True, net=None):
    """z = omega D^-1 r + P net(R r), with the input scaled to rms(r) = 1 over the free cells"""
    r = np.asarray(r, dtype=np.float64).reshape(fine)
    ex = excluded_mask(fine, pin, solid)
    nfree = (~ex).sum()
    rr = float((r * r).sum())
    sc = np.sqrt(nfree / rr) if rr > 0 else 0.0
    dims = level_dims(fine)
    net = net or UNet(params, fine, rounding)
    y = net.forward(restrict(r, fine, dims[0]) * sc)
    d = diag_B(fine, solid)
    jac = np.where(d > 0, r / np.maximum(d, 1), 0.0)
    z = params[-1] * jac + prolong(y, fine) / (sc if sc > 0 else 1.0)
    z[ex] = 0.0
    return z


def loss_and_grad(params, r, p, fine, pin, solid=None, rounding=True):
    """energy-norm loss of the preconditioner on a normalised pair and its parameter gradient"""
    r = np.asarray(r, dtype=np.float64).reshape(fine)
    p = np.asarray(p, dtype=np.float64).reshape(fine)
    dims = level_dims(fine)
    net = UNet(params, fine, rounding)
    y = net.forward(restrict(r, fine, dims[0]))
    d = diag_B(fine, solid)
    jac = np.where(d > 0, r / np.maximum(d, 1), 0.0)
    ex = excluded_mask(fine, pin, solid)
    z = params[-1] * jac + prolong(y, fine)
    z[ex] = 0.0
    e = z - p
    e[ex] = 0.0
    Be = apply_B(e, fine, pin, solid)
    denom = float((p * apply_B(p, fine, pin, solid)).sum())
    loss = float((e * Be).sum()) / denom
    gz = 2.0 * Be / denom
    gz[ex] = 0.0
    gp = net.backward(prolong_adjoint(gz, dims[0]))
    gp[-1] = float((gz * jac).sum())
    return loss, gp


def normalise_pair(r, p, fine, pin, solid=None):
    ex = excluded_mask(fine, pin, solid)
    nfree = (~ex).sum()
    r = np.asarray(r, dtype=np.float64).reshape(fine)
    s = np.sqrt(nfree / float((r * r).sum()))
    return r * s, np.asarray(p, dtype=np.float64).reshape(fine) * s


def init_params(seed=1):
    """He-normal weights (std sqrt(2 / (27 cin)); the linear output layer sqrt(1 / (27 cin))), omega 2/3."""
    rng = np.random.default_rng(seed)
    out = []
    for lev, cin, cout, relu, *_ in LAYERS:
        out.append(rng.normal(0.0, np.sqrt((2.0 if relu else 1.0) / (27 * cin)), size=27 * cin * cout))
    out.append([2.0 / 3.0])
    return np.concatenate(out).astype(np.float32)
