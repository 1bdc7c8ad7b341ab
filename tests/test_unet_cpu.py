"""CPU pins of the network oracle (oracle/unet_oracle.py): its forward pass and its
hand-written backward pass against torch autograd on the same FP64 network, and its
bfloat16 rounding against torch's."""
import numpy as np
import pytest

from oracle import unet_oracle as U

torch = pytest.importorskip("torch")
F = torch.nn.functional


def torch_net(p, inp, target, c=16):
    L = U.layout(c)
    n = round(inp.shape[0] ** (1 / 3))
    P = torch.tensor(p, dtype=torch.float64, requires_grad=True)
    Ws, bs = [], []
    for l in range(U.NCONV):
        co, ci = L["cout"][l], L["cin"][l]
        w = P[L["woff"][l]:L["woff"][l] + 27 * co * ci].reshape(3, 3, 3, co, ci).permute(3, 4, 0, 1, 2)
        Ws.append(w)
        bs.append(P[L["boff"][l]:L["boff"][l] + co])
    hw = P[L["hw"]:L["hw"] + 4 * c].reshape(4, c)
    hb = P[L["hb"]:L["hb"] + 4]
    x = torch.zeros(1, U.IN_CH, n, n, n, dtype=torch.float64)
    x[0, :U.IN_USED] = torch.tensor(inp, dtype=torch.float64).reshape(n, n, n, U.IN_USED).permute(3, 0, 1, 2)

    def cv(l, a):
        return F.relu(F.conv3d(a, Ws[l], bs[l], padding=1))

    up = lambda a: F.interpolate(a, scale_factor=2, mode="nearest")
    a0 = cv(0, x)
    s0 = cv(1, a0)
    a1 = cv(2, F.avg_pool3d(s0, 2))
    s1 = cv(3, a1)
    a2 = cv(4, F.avg_pool3d(s1, 2))
    b2 = cv(5, a2)
    b1d = cv(7, cv(6, torch.cat([up(b2), s1], 1)))
    b0d = cv(9, cv(8, torch.cat([up(b1d), s0], 1)))
    out = torch.einsum("bcijk,oc->bijko", b0d, hw) + hb
    t = torch.tensor(target, dtype=torch.float64).reshape(1, n, n, n, 4)
    loss = ((out - t) ** 2).sum() / (t ** 2).sum()
    loss.backward()
    return out.detach().numpy().reshape(-1, 4), float(loss.detach()), P.grad.numpy()


def random_case(n, seed):
    rng = np.random.default_rng(seed)
    L = U.layout()
    p = np.zeros(L["nparam"])
    for l in range(U.NCONV):
        fan = 27 * L["cin"][l]
        p[L["woff"][l]:L["boff"][l]] = rng.uniform(-1, 1, L["boff"][l] - L["woff"][l]) * np.sqrt(6 / fan)
        p[L["boff"][l]:L["boff"][l] + L["cout"][l]] = rng.uniform(-0.1, 0.1, L["cout"][l])
    p[L["hw"]:L["kappa"]] = rng.uniform(-0.5, 0.5, L["kappa"] - L["hw"])
    p[L["kappa"]] = 1.0
    inp = rng.normal(size=(n ** 3, U.IN_USED))
    tgt = rng.normal(size=(n ** 3, 4))
    return p, inp, tgt


@pytest.mark.parametrize("n", [8, 12])
def test_oracle_matches_torch_autograd(n):
    p, inp, tgt = random_case(n, 7 + n)
    ref_out, ref_loss, ref_grad = torch_net(p, inp, tgt)
    r = U.forward_backward(p, inp, tgt, bf=False)
    assert np.allclose(r["out"], ref_out, rtol=1e-10, atol=1e-12)
    assert abs(r["loss"] - ref_loss) <= 1e-12 * abs(ref_loss)
    L = U.layout()
    g = r["grad"]
    # every parameter block, kappa excluded (not part of the loss)
    assert g[L["kappa"]] == 0 and ref_grad[L["kappa"]] == 0
    assert np.allclose(g, ref_grad, rtol=1e-9, atol=1e-13)
    assert np.linalg.norm(g) > 0


def test_bf16_rounding_matches_torch():
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.normal(size=4000).astype(np.float32) * 10.0 ** rng.integers(-6, 6, 4000),
                        np.array([0.0, -0.0, 1.0, 1.00390625, 1.0078125, 1.005859375, 3.0e38], np.float32)])
    ref = torch.tensor(x).to(torch.bfloat16).to(torch.float32).numpy()
    assert np.array_equal(U.bf16(x), ref)


def test_adam_restatement():
    rng = np.random.default_rng(1)
    p = rng.normal(size=50)
    g = rng.normal(size=50)
    P = torch.tensor(p[:-1].copy(), requires_grad=True)
    opt = torch.optim.Adam([P], lr=1e-3, betas=(0.9, 0.999), eps=1e-8)
    m = np.zeros(50)
    v = np.zeros(50)
    q = p.copy()
    for t in range(1, 4):
        P.grad = torch.tensor(g[:-1] * t)
        opt.step()
        q, m, v = U.adam(q, g * t, m, v, t, 1e-3)
    assert np.allclose(q[:-1], P.detach().numpy(), rtol=1e-12, atol=1e-14)
    assert q[-1] == p[-1]
