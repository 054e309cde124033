"""The network oracle's analytic gradient against central finite differences
(FP64, no BF16 rounding), so the GPU gradients are checked against a pinned
reference."""
import numpy as np

from oracle import mpnn_oracle as mo


def _graph(F, rng):
    adj = [set() for _ in range(F)]
    for e in range(F):
        for q in rng.choice(F, 4, replace=False):
            if q != e:
                adj[e].add(int(q))
                adj[int(q)].add(e)
    W = max(len(a) for a in adj)
    nbr = np.tile(np.arange(F)[:, None], (1, W))
    for e in range(F):
        lst = sorted(adj[e])
        nbr[e, :len(lst)] = lst
    return nbr, np.array([len(a) for a in adj])


def test_finite_differences():
    rng = np.random.default_rng(0)
    F = 40
    nbr, deg = _graph(F, rng)
    x = rng.standard_normal((F, mo.FIN))
    y = rng.standard_normal(F)
    mask = np.ones(F)
    mask[:4] = 0
    p = mo.init_params(1)
    for k in p:
        p[k] = p[k] + 0.05 * rng.standard_normal(p[k].shape)
    _, g, _ = mo.loss_and_grads(p, x, nbr, deg, y, mask, bf=False)
    worst = 0.0
    for k in p:
        for _ in range(3):
            idx = tuple(int(rng.integers(0, s)) for s in p[k].shape)
            eps = 1e-6
            pp = {a: b.copy() for a, b in p.items()}
            pm = {a: b.copy() for a, b in p.items()}
            pp[k][idx] += eps
            pm[k][idx] -= eps
            lp, _, _ = mo.loss_and_grads(pp, x, nbr, deg, y, mask, bf=False)
            lm, _, _ = mo.loss_and_grads(pm, x, nbr, deg, y, mask, bf=False)
            fd = (lp - lm) / (2 * eps)
            worst = max(worst, abs(fd - g[k][idx]) / max(abs(fd), 1e-8))
    assert worst < 1e-5


def test_bf16_rounding():
    v = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 65504.0, 1e-40])
    r = mo.bf16(v)
    # BF16 keeps 8 significant bits
    assert np.all(np.abs(r - v) <= np.abs(v) * 2.0 ** -8 + 1e-38)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125
