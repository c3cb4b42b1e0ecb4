"""The numpy restatement of the warm-start network (the checker of the CUDA
training kernels): its backpropagated gradients against central finite
differences, in float64."""
import numpy as np

import mpnn_np as MP


def _problem(seed=0, n=12, hidden=5, layers=2):
    rng = np.random.default_rng(seed)
    shapes = [((hidden, 6), hidden)] + [((hidden, 2 * hidden), hidden)] * layers + [((3, hidden), 3)]
    params = [(rng.standard_normal(ws) * 0.5, rng.standard_normal(bs) * 0.1) for ws, bs in shapes]
    # ring graph with chords, mean aggregation
    rows = [sorted({(i - 1) % n, (i + 1) % n, (i + 5) % n}) for i in range(n)]
    ptr = np.concatenate([[0], np.cumsum([len(r) for r in rows])])
    col = np.concatenate(rows)
    wt = np.concatenate([[1.0 / len(r)] * len(r) for r in rows])
    A = MP.adjacency(n, ptr, col, wt)
    x = rng.standard_normal((n, 6))
    t = rng.standard_normal((n, 3))
    return params, x, A, t


def test_gradients_match_finite_differences():
    params, x, A, t = _problem()
    _, _, grads = MP.loss_and_grads(params, x, A, t)
    h = 1e-6
    rng = np.random.default_rng(1)
    for li, (W, b) in enumerate(params):
        for arr, g in ((W, grads[li][0]), (b, grads[li][1])):
            for _ in range(6):
                idx = tuple(rng.integers(0, s) for s in arr.shape)
                old = arr[idx]
                arr[idx] = old + h
                lp = MP.loss_and_grads(params, x, A, t)[0]
                arr[idx] = old - h
                lm = MP.loss_and_grads(params, x, A, t)[0]
                arr[idx] = old
                fd = (lp - lm) / (2 * h)
                assert abs(fd - g[idx]) <= 1e-6 + 1e-5 * abs(fd), (li, idx, fd, g[idx])


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.140625, 1e-20], np.float32)
    r = MP.bf16_round(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125 and r[3] == -3.140625
    assert np.all((r.view(np.uint32) & 0xFFFF) == 0)
