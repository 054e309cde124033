"""Learned warm start on the GPU (tcgen05 BF16 kernels) vs the CPU oracle.

* forward: the GPU network output equals the oracle's (FP64 with BF16
  rounding at the same points) within BF16 accuracy;
* gradients: every parameter tensor's gradient from the GPU backward kernels
  matches the oracle's analytic gradient (which tests/test_mpnn_oracle.py
  checks against finite differences);
* training: the online-trained network lowers the FP64 BiCGStab iteration
  count against the previous-step warm start, while the solution stays the
  plain FP64 form's (same tolerance).
"""
import numpy as np
import pytest

from helpers import rel_err
from mhfem import _lib as L
from mhfem import problems
from oracle import mpnn_oracle as mo

pytestmark = pytest.mark.gpu


def flatten(p):
    parts = [p["W0"], p["b0"]]
    for l in range(1, mo.LAYERS + 1):
        parts += [p[f"W{l}"], p[f"b{l}"]]
    parts += [p["wd"], p["bd"]]
    return np.concatenate([np.asarray(x, np.float64).ravel() for x in parts]).astype(np.float32)


def unflatten(v):
    out, o = {}, 0
    shapes = [("W0", (mo.FIN, mo.H)), ("b0", (mo.H,))]
    for l in range(1, mo.LAYERS + 1):
        shapes += [(f"W{l}", (2 * mo.H, mo.H)), (f"b{l}", (mo.H,))]
    shapes += [("wd", (mo.H,)), ("bd", (1,))]
    for name, shp in shapes:
        n = int(np.prod(shp))
        out[name] = np.asarray(v[o:o + n], np.float64).reshape(shp)
        o += n
    return out


def graph_from_solver(s):
    rowptr, cols, _, _ = s.system()
    F = s.F
    W = int(np.diff(rowptr).max()) - 1
    nbr = np.tile(np.arange(F)[:, None], (1, W))
    deg = np.zeros(F, np.int64)
    for r in range(F):
        c = [x for x in cols[rowptr[r]:rowptr[r + 1]] if x != r]
        nbr[r, :len(c)] = c
        deg[r] = len(c)
    return nbr, deg


@pytest.fixture(scope="module")
def small():
    p = problems.diffusion3d(N=4, steps=1, form=L.FORM_LEARNED)
    s = problems.make_solver(p)
    nbr, deg = graph_from_solver(s)
    fv, fc, _ = s.topology()
    tags, _, _ = p.bc_fn(fv, fc)
    fixed = (fc[:, 1] < 0) & (tags == 0)
    rng = np.random.default_rng(3)
    x = rng.standard_normal((s.F, 16)).astype(np.float32)
    params = mo.init_params(5)
    for k in params:
        params[k] = params[k] + 0.05 * rng.standard_normal(params[k].shape)
    # round-trip through float32 so both sides start from identical values
    params = unflatten(flatten(params))
    s.set_learned_params(flatten(params))
    yield s, nbr, deg, fixed, x, params
    s.close()


def test_learned_params_roundtrip(small):
    s, *_, params = small
    assert np.array_equal(s.learned_params(), flatten(params))


def test_forward_matches_oracle(small):
    s, nbr, deg, fixed, x, params = small
    out = s.learned_forward(x)
    ref, _ = mo.forward(params, x.astype(np.float64), nbr, deg, bf=True)
    assert np.abs(out - ref).max() < 2e-2 * np.abs(ref).max()
    ref64, _ = mo.forward(params, x.astype(np.float64), nbr, deg, bf=False)
    assert np.abs(out - ref64).max() < 5e-2 * np.abs(ref64).max()


def test_gradients_match_oracle(small):
    """The GPU's gradients against the oracle's, which rounds to BF16 at the
    same points (dZ, the neighbour-mean gradients, the activations).  What is
    left is where the two round FP32 and FP64 sums of the same terms to
    different BF16 neighbours: one BF16 step is 2^-8 = 3.9e-3 of a value,
    and such flips compound from the top layer down; measured on 864 and
    6,528 faces, the top layer's gradients agree to 1e-5, W2 to 5e-3..1.1e-2
    and the encoder's W0 to 1.4e-2..3.1e-2, hence the 5e-2 bound (13 BF16
    steps)."""
    s, nbr, deg, fixed, x, params = small
    rng = np.random.default_rng(9)
    y = rng.standard_normal(s.F)
    loss, g = s.learned_gradients(x, y)
    mask = (~fixed).astype(np.float64)
    loss_ref, g_ref, _ = mo.loss_and_grads(params, x.astype(np.float64), nbr, deg, y, mask, bf=True)
    assert abs(loss - loss_ref) < 1e-2 * loss_ref
    gg = unflatten(g)
    for k in g_ref:
        err = np.linalg.norm(gg[k] - g_ref[k]) / max(np.linalg.norm(g_ref[k]), 1e-30)
        assert err < 5e-2, f"gradient {k}: relative error {err:.3e}"


def _assert_gate_picked_the_lowest_residual(st):
    """The solve started from the candidate with the lowest relative residual
    among the warm start, the extrapolated base and the network's guess
    (each present when it was formed)."""
    cand = {0: st["warm_residual"]}
    if st["base_residual"] > 0:
        cand[2] = st["base_residual"]
    if st["guess_residual"] > 0:
        cand[1] = st["guess_residual"]
    assert st["guess_source"] in cand
    assert cand[st["guess_source"]] <= min(cand.values()), (st["guess_source"], cand)


def test_learned_warm_start_reduces_iterations():
    """Online training on 40 method-generated steps of the time-varying source
    problem, then 20 steps where the network's guess competes with the
    previous-step warm start; the plain FP64 form runs the same steps."""
    N, train, use = 12, 40, 20
    steps = train + use
    pl = problems.diffusion3d_source(N=N, steps=steps, form=L.FORM_LEARNED)
    pl.source = (0.5, 60 * pl.dt)
    sl = problems.make_solver(pl)
    sl.learned_options(train_steps=train, train_iters=4, learning_rate=2e-3)
    pf = problems.diffusion3d_source(N=N, steps=steps, form=L.FORM_FP64)
    pf.source = pl.source
    sf = problems.make_solver(pf)
    it_l, it_f, used = [], [], 0
    t = 0.0
    for k in range(steps):
        a = sl.step(t, pl.dt)
        b = sf.step(t, pf.dt)
        if k >= 1:
            _assert_gate_picked_the_lowest_residual(a)
        if k >= train:
            it_l.append(a["iterations"])
            it_f.append(b["iterations"])
            used += a["guess_used"]
        t += pl.dt
    st = sl.learned_status()
    assert st["trained_steps"] == train
    zl, _ = sl.state()
    zf, _ = sf.state()
    assert rel_err(zl, zf) < 1e-7  # both solved to the same 1e-10 tolerance
    assert np.mean(it_l) < 0.9 * np.mean(it_f), (np.mean(it_l), np.mean(it_f))
    sl.close()
    sf.close()


def test_learned_guess_with_mixed_solve():
    """A network trained on one solver, loaded into a second one whose solve
    from the guess is the mixed-precision refinement: the guess is used, the
    FP64 residual meets the tolerance in every step, the traces agree with
    the plain FP64 form, and the inner FP32 iterations fall below those of
    the mixed form started from the previous step."""
    N, train, use = 12, 40, 12
    src = (0.5, 60 * 1e-3)
    pl = problems.diffusion3d_source(N=N, steps=train + use, form=L.FORM_LEARNED)
    pl.source = src
    sl = problems.make_solver(pl)
    sl.learned_options(train_steps=train, train_iters=4, learning_rate=2e-3)
    t = 0.0
    for _ in range(train):
        sl.step(t, pl.dt)
        t += pl.dt
    zf0, zk0 = sl.state()
    params = sl.learned_params()
    sl.close()

    def make(form):
        p = problems.diffusion3d_source(N=N, steps=train + use, form=form)
        p.source = src
        s = problems.make_solver(p)
        s.setInitialCondition(zk0, zf0)
        return p, s

    pm, sm = make(L.FORM_LEARNED)
    sm.learned_options(train_steps=0, mixed_solve=True)
    sm.set_learned_params(params)
    pmx, smx = make(L.FORM_MIXED)
    pf, sf = make(L.FORM_FP64)
    inner_l, inner_m, used = [], [], 0
    for k in range(use):
        a = sm.step(t, pl.dt)
        b = smx.step(t, pl.dt)
        sf.step(t, pl.dt)
        assert a["residual"] < pl.tol and a["sweeps"] >= 1
        if k >= 1:  # the first step has no history for the network's features
            _assert_gate_picked_the_lowest_residual(a)
            inner_l.append(a["iterations"])
            inner_m.append(b["iterations"])
            used += a["guess_used"]
        t += pl.dt
    zl, _ = sm.state()
    zf, _ = sf.state()
    assert rel_err(zl, zf) < 1e-7
    assert np.mean(inner_l) < np.mean(inner_m), (np.mean(inner_l), np.mean(inner_m))
    for s in (sm, smx, sf):
        s.close()


def test_network_gain_over_the_extrapolation_alone():
    """What the trained network adds to the method without it: on the linear
    extrapolation base (2 Zn - Zn1, the previous two traces) the network's
    correction wins the gate in some steps after training and the solves
    need no more iterations than with the base alone.  (On the cubic base
    the extrapolation is so close that the network's correction rarely wins;
    the benchmark reports both.)"""
    N, train, use = 12, 40, 20
    src = (0.5, 60 * 1e-3)
    runs = {}
    for name, train_steps in (("net", train), ("base_only", 0)):
        p = problems.diffusion3d_source(N=N, steps=train + use, form=L.FORM_LEARNED)
        p.source = src
        s = problems.make_solver(p)
        s.learned_options(train_steps=train_steps, train_iters=4, learning_rate=2e-3, extrapolation_order=1)
        its, won = [], 0
        t = 0.0
        for k in range(train + use):
            st = s.step(t, p.dt)
            if k >= 1:
                _assert_gate_picked_the_lowest_residual(st)
            if k >= train:
                its.append(st["iterations"])
                won += st["guess_source"] == 1
            t += p.dt
        runs[name] = (np.mean(its), won, s.state()[0])
        s.close()
    assert runs["base_only"][1] == 0
    assert runs["net"][1] >= 1, runs["net"][:2]
    assert runs["net"][0] <= runs["base_only"][0] + 1.0, (runs["net"][0], runs["base_only"][0])
    assert rel_err(runs["net"][2], runs["base_only"][2]) < 1e-7
