"""CPU checks of the proposal network's oracle: its analytic gradient
against finite differences (float64, no bf16 rounding), on a small input."""
import numpy as np

from oracle import cnn_oracle as CO


def _small_problem(seed=0, S=16):
    rng = np.random.default_rng(seed)
    occ = (rng.random((2, S, S)) < 0.2).astype(np.float64) * 0.5
    ev = S // 4
    geos = [(4.0 * 2, -30.0, 128 / 61.0, ev, ev), (8.0, -25.0, 128 / 51.0, ev, ev - 1)]
    p = rng.standard_normal(CO.n_params()) * 0.15
    p[-2], p[-1] = 0.8, -1.0
    target = (rng.random((2, CO.HEAD_T, CO.HEAD_R)) < 0.01).astype(np.float64)
    return occ, geos, p, target


def test_layer_count_and_parameters():
    assert len(CO.LAYERS) == 6 and all(c in (1, 32) for l in CO.LAYERS for c in l[:2])
    assert CO.n_params() == 288 + 32 + 4 * (9216 + 32) + 288 + 1 + 2


def test_gradient_matches_finite_differences():
    occ, geos, p, target = _small_problem()
    loss, g = CO.net_loss_grads(occ, geos, p, target, 20.0, exact=True)
    rng = np.random.default_rng(1)
    idx = list(rng.choice(CO.n_params() - 2, 12, replace=False)) + [CO.n_params() - 2,
                                                                    CO.n_params() - 1]
    for i in idx:
        h = 1e-6 * max(1.0, abs(p[i]))
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        lp, _ = CO.net_loss_grads(occ, geos, pp, target, 20.0, exact=True)
        lm, _ = CO.net_loss_grads(occ, geos, pm, target, 20.0, exact=True)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-5 + 1e-3 * abs(fd), (i, fd, g[i])
