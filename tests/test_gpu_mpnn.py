"""Warm-start network on the GPU: the CUDA forward and backward kernels
against the numpy oracle (tolerances for float32 accumulation against
float64), bitwise reproducible training, and what the trained network gains:
fewer steps to steady state than the uniform start on held-out geometries."""
import numpy as np
import pytest

import mpnn_np as MP

pytestmark = pytest.mark.gpu


def _random_sample(n=300, seed=0):
    """A random graph with layers of both kinds: mesh-like neighbour means
    (layers 1, 2), count-aware bins on a 5 x 5 grid (layer 3) and bin means
    on a 2 x 2 grid (layer 4)."""
    from fvdbm_jax_gb300.warmstart import NFEAT, Sample, _stage, grid_mean
    rng = np.random.default_rng(seed)
    # random planar-ish graph: ring plus random chords, symmetric, mean weights
    nbr = [set() for _ in range(n)]
    for i in range(n):
        for j in ((i + 1) % n, int(rng.integers(0, n))):
            if j != i:
                nbr[i].add(j)
                nbr[j].add(i)
    import scipy.sparse as sp
    rows = np.concatenate([[i] * len(s) for i, s in enumerate(nbr)])
    cols = np.concatenate([sorted(s) for s in nbr])
    M = sp.csr_matrix((np.ones(rows.size), (rows, cols)), shape=(n, n))
    deg = np.asarray(M.sum(1)).reshape(-1)
    A = (sp.diags(1.0 / deg) @ M).tocsr().astype(np.float32)
    xy = rng.uniform(0, 1, (n, 2))
    P5, U5 = grid_mean(xy, 5, counted=True)
    P2, U2 = grid_mean(xy, 2)
    aggs = [[_stage(A)], [_stage(A)], [_stage(P5), _stage(U5)], [_stage(P2), _stage(U2)]]
    dense = [A.toarray()] * 2 + [(U5.astype(np.float32) @ P5.astype(np.float32)).toarray(),
                                 (U2.astype(np.float32) @ P2.astype(np.float32)).toarray()]
    x = rng.standard_normal((n, NFEAT)).astype(np.float32)
    t = rng.standard_normal((n, 3)).astype(np.float32)
    return Sample(x, aggs, t), [d.astype(np.float64) for d in dense]


def test_forward_backward_match_oracle():
    from fvdbm_jax_gb300.warmstart import MPNN
    smp, A = _random_sample()
    net = MPNN(seed=3, scales=("mesh", "mesh", "c5", 2))
    g = net._upload([smp], True)  # identity feature/target scaling
    loss = float(net.loss_and_grads(g).item())
    y = g["y"].detach().cpu().numpy()
    params = net.get_params(rounded=True)
    lo, yo, go = MP.loss_and_grads(params, smp.x, A, smp.t)
    assert abs(loss - lo) <= 1e-5 * lo
    assert np.allclose(y, yo, rtol=1e-4, atol=1e-4)
    for (gw, gb), (ow, ob) in zip(net.grads(), go):
        scale = max(np.abs(ow).max(), 1e-6)
        assert np.abs(gw - ow).max() <= 1e-4 * scale, (np.abs(gw - ow).max(), scale)
        assert np.abs(gb - ob).max() <= 1e-4 * max(np.abs(ob).max(), 1e-6)


def test_training_is_reproducible_and_learns():
    from fvdbm_jax_gb300.warmstart import MPNN
    smp, _ = _random_sample(n=500, seed=5)
    # a learnable target: a smooth function of the features
    smp.t = np.stack([np.tanh(smp.x[:, 0]), smp.x[:, 1] * smp.x[:, 2] * 0.3, np.sin(smp.x[:, 3])], 1).astype(
        np.float32)
    hists, params = [], []
    for _ in range(2):
        net = MPNN(seed=11, scales=("mesh", "mesh", "c5", 2))
        hists.append(net.fit([smp], epochs=300, lr=3e-3, log_every=50))
        params.append(net.get_params(rounded=False))
    assert hists[0] == hists[1]
    for (a, b), (c, d) in zip(*params):
        assert np.array_equal(a, c) and np.array_equal(b, d)
    assert hists[0][-1][1] < 0.2 * hists[0][0][1]


def test_warm_start_needs_fewer_steps_than_uniform():
    from fvdbm_jax_gb300 import Batch
    from fvdbm_jax_gb300 import cases as CS
    from fvdbm_jax_gb300 import warmstart as WS
    rng = np.random.default_rng(7)

    def make(k):
        rin, rout = float(rng.uniform(1.01, 1.05)), float(rng.uniform(0.95, 0.99))
        case = CS.porous_square(int(rng.integers(6, 16)), int(rng.uniform(1500, 3000)), 0.65, rho_in=rin,
                                rho_out=rout, porosity=0.8, delta_t=1.0, seed=1000 + k, mesher=True)
        return case, rin, rout

    train = [make(k) for k in range(24)]
    test = [make(100 + k) for k in range(6)]
    thr, every, cap = 1e-6, 100, 60_000
    b = Batch([c[0][1:4] for c in train])
    b.init()
    steps, res, status = b.run_to_steady(thr, every, cap)
    st = b.state()
    samples = []
    for s, (case, rin, rout) in enumerate(train):
        cs = b.case_state(s, st)
        rho, vel = WS.macros(cs["pdf"])
        samples.append(WS.sample(case, rin, rout, rho, vel))
    b.close()
    net = WS.MPNN(seed=0)
    hist = net.fit(samples, epochs=600, lr=3e-3, log_every=100)
    assert hist[-1][1] < hist[0][1]
    # held-out: uniform start against the predicted start, same solver and loop
    plain = Batch([c[0][1:4] for c in test])
    plain.init()
    sp_, stp, _ = WS.run_cases(plain, thr, every, cap)
    warm = Batch([c[0][1:4] for c in test])
    warm.init()
    rho, vel = [], []
    for case, rin, rout in test:
        y = net.predict(WS.sample(case, rin, rout))
        r, v = WS.untarget(y, rin, rout)
        rho.append(r)
        vel.append(v)
    sw, stw, restarted = WS.run_cases(warm, thr, every, cap, init=(np.concatenate(rho), np.concatenate(vel)))
    assert np.all(stp == 1) and np.all(stw == 1), (stp, stw)
    assert sw.sum() < sp_.sum(), (sw, sp_)
