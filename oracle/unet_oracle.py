"""CPU restatement of the learned preconditioner's network (TEST INFRASTRUCTURE ONLY).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` import
this module; the product library never does.  The network has no counterpart in the
reference (the reference has no learned component), so its oracle is this numpy
restatement, pinned against torch autograd on the CPU (tests/test_unet_cpu.py).

Layout (the C ABI's, stg_net_* in include/stokes_gb300.h):
  * grid n^3, cell v = (i n + j) n + k, channel-last arrays [n, n, n, C];
  * parameters one float vector: per convolution l the weights [27][C_out][C_in] with tap
    t = 9 (di+1) + 3 (dj+1) + (dk+1), then the biases [C_out]; the 1x1 head [4][c] and [4];
    last the output scale kappa;
  * convolution l reads x[v + (di, dj, dk)] with zero padding (cross-correlation).

``bf16=True`` rounds, as the GPU path does, the input, every stored activation, the
convolution weights and every ReLU-masked gradient to bfloat16 (round to nearest even);
accumulation is FP64 here (FP32 on the GPU).  ``bf16=False`` is the exact FP64 network.
"""
import numpy as np

IN_CH = 16
IN_USED = 8
OUT_CH = 4
NCONV = 10


def layout(c=16):
    cin = [IN_CH, c, c, 2 * c, 2 * c, 4 * c, 6 * c, 2 * c, 3 * c, c]
    cout = [c, c, 2 * c, 2 * c, 4 * c, 4 * c, 2 * c, 2 * c, c, c]
    off = 0
    woff, boff = [], []
    for l in range(NCONV):
        woff.append(off)
        off += 27 * cout[l] * cin[l]
        boff.append(off)
        off += cout[l]
    hw = off
    off += OUT_CH * c
    hb = off
    off += OUT_CH
    kappa = off
    off += 1
    return dict(c=c, cin=cin, cout=cout, woff=woff, boff=boff, hw=hw, hb=hb, kappa=kappa, nparam=off)


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (u & 0xFFFFFFFF).astype(np.uint32).view(np.float32).reshape(a.shape)


def unpack(p, L):
    """Parameter vector -> (list of W[27][co][ci], list of b[co], head W[4][c], head b[4])."""
    W = [p[L["woff"][l]:L["woff"][l] + 27 * L["cout"][l] * L["cin"][l]].reshape(27, L["cout"][l], L["cin"][l])
         for l in range(NCONV)]
    b = [p[L["boff"][l]:L["boff"][l] + L["cout"][l]] for l in range(NCONV)]
    hw = p[L["hw"]:L["hw"] + OUT_CH * L["c"]].reshape(OUT_CH, L["c"])
    hb = p[L["hb"]:L["hb"] + OUT_CH]
    return W, b, hw, hb


def taps():
    return [(t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1) for t in range(27)]


def shifted(x, d):
    """y[v] = x[v + d] with zero padding (x: [n, n, n, C])."""
    n = x.shape[0]
    y = np.zeros_like(x)
    src = [slice(max(0, s), n + min(0, s)) for s in d]
    dst = [slice(max(0, -s), n - max(0, s)) for s in d]
    y[dst[0], dst[1], dst[2]] = x[src[0], src[1], src[2]]
    return y


def conv(x, W, b):
    y = np.zeros(x.shape[:3] + (W.shape[1],))
    for t, d in enumerate(taps()):
        y += shifted(x, d) @ W[t].T
    return y + b


def conv_dx(dy, W):
    """Input gradient: dx[v] = sum_t dy[v - o_t] W[t]."""
    dx = np.zeros(dy.shape[:3] + (W.shape[2],))
    for t, (a, b_, c) in enumerate(taps()):
        dx += shifted(dy, (-a, -b_, -c)) @ W[t]
    return dx


def conv_dw(x, dy):
    """dW[t][co][ci] = sum_v dy[v][co] x[v + o_t][ci]."""
    C_in, C_out = x.shape[3], dy.shape[3]
    dW = np.zeros((27, C_out, C_in))
    dyf = dy.reshape(-1, C_out)
    for t, d in enumerate(taps()):
        dW[t] = dyf.T @ shifted(x, d).reshape(-1, C_in)
    return dW


def pool(x):
    n = x.shape[0] // 2
    return x.reshape(n, 2, n, 2, n, 2, -1).sum(axis=(1, 3, 5)) * 0.125


def pool_bwd(g):
    return np.repeat(np.repeat(np.repeat(g, 2, 0), 2, 1), 2, 2) * 0.125


def up(x):
    return np.repeat(np.repeat(np.repeat(x, 2, 0), 2, 1), 2, 2)


def up_bwd(g):
    n = g.shape[0] // 2
    return g.reshape(n, 2, n, 2, n, 2, -1).sum(axis=(1, 3, 5))


def forward_backward(params, inp, target=None, bf=True, c=16):
    """inp [n^3][8] (float), target [n^3][4] or None.

    Returns dict(out [n^3][4], loss, grad [nparam]) (loss / grad only with a target). The
    loss is the relative squared error sum (out - target)^2 / sum target^2."""
    L = layout(c)
    p = np.asarray(params, dtype=np.float64)
    W, b, hw, hb = unpack(p, L)
    r = (lambda a: bf16(a).astype(np.float64)) if bf else (lambda a: np.asarray(a, dtype=np.float64))
    Wr = [r(w) for w in W]
    V = inp.shape[0]
    n = round(V ** (1.0 / 3.0))
    x0 = np.zeros((n, n, n, IN_CH))
    x0[..., :IN_USED] = (r(np.asarray(inp, dtype=np.float32)) if bf else np.asarray(inp, np.float64)).reshape(n, n, n, IN_USED)

    def cv(l, x):
        return r(np.maximum(conv(x, Wr[l], b[l]), 0.0))

    a0 = cv(0, x0)
    s0 = cv(1, a0)
    p0 = r(pool(s0))
    a1 = cv(2, p0)
    s1 = cv(3, a1)
    p1 = r(pool(s1))
    a2 = cv(4, p1)
    b2 = cv(5, a2)
    cat1 = np.concatenate([up(b2), s1], axis=3)
    a1d = cv(6, cat1)
    b1d = cv(7, a1d)
    cat0 = np.concatenate([up(b1d), s0], axis=3)
    a0d = cv(8, cat0)
    b0d = cv(9, a0d)
    out = b0d @ hw.T + hb
    res = {"out": out.reshape(V, OUT_CH)}
    if target is None:
        return res
    t = np.asarray(target, dtype=np.float64).reshape(n, n, n, OUT_CH)
    t2 = float(np.sum(t ** 2))
    res["loss"] = float(np.sum((out - t) ** 2) / t2)
    dout = 2.0 * (out - t) / t2
    g = np.zeros(L["nparam"])

    def put(l, dW, db):
        g[L["woff"][l]:L["woff"][l] + dW.size] = dW.ravel()
        g[L["boff"][l]:L["boff"][l] + db.size] = db

    g[L["hw"]:L["hw"] + OUT_CH * c] = (dout.reshape(-1, OUT_CH).T @ b0d.reshape(-1, c)).ravel()
    g[L["hb"]:L["hb"] + OUT_CH] = dout.reshape(-1, OUT_CH).sum(0)
    G = dout @ hw

    def back(l, gy, y, x, need_dx=True):
        dy = r(np.where(y > 0, gy, 0.0))
        put(l, conv_dw(x, dy), dy.reshape(-1, dy.shape[3]).sum(0))
        return conv_dx(dy, Wr[l]) if need_dx else None

    G = back(9, G, b0d, a0d)
    Gcat0 = back(8, G, a0d, cat0)
    G = up_bwd(Gcat0[..., :2 * c])
    G = back(7, G, b1d, a1d)
    Gcat1 = back(6, G, a1d, cat1)
    G = up_bwd(Gcat1[..., :4 * c])
    G = back(5, G, b2, a2)
    G = back(4, G, a2, p1)
    Gs1 = Gcat1[..., 4 * c:] + pool_bwd(G)
    G = back(3, Gs1, s1, a1)
    G = back(2, G, a1, p0)
    Gs0 = Gcat0[..., 2 * c:] + pool_bwd(G)
    G = back(1, Gs0, s0, a0)
    back(0, G, a0, x0, need_dx=False)
    res["grad"] = g
    return res


def adam(p, g, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step on all parameters but the last (kappa); returns new (p, m, v)."""
    p, m, v = p.copy(), m.copy(), v.copy()
    k = len(p) - 1
    m[:k] = b1 * m[:k] + (1 - b1) * g[:k]
    v[:k] = b2 * v[:k] + (1 - b2) * g[:k] ** 2
    p[:k] = p[:k] - lr * (m[:k] / (1 - b1 ** t)) / (np.sqrt(v[:k] / (1 - b2 ** t)) + eps)
    return p, m, v
