"""CPU checks of the selector tooling: feature layout, weight layout, and
that training fits a cost table it can then choose from."""

import numpy as np

from dawn_gb300 import abi, selector as S


def test_weight_layout_matches_the_abi():
    assert S.N_WEIGHTS == abi.SELECTOR_WEIGHTS == 1475
    rng = np.random.default_rng(0)
    p = S.init_params(rng)
    w = S.flatten(p)
    q = S.unflatten(w)
    for a, b in zip(p, q):
        assert np.allclose(a, b, atol=1e-6)


def test_features_are_normalised():
    x = S.features(1 << 22, 1.28e8, [1, 1000, 2e6], [16, 1e5, 1e8], [1e8, 5e7, 1e3], [2, 3, 9], [1, 1, 1000], 64)
    assert x.shape == (3, S.N_IN)
    assert np.all(x >= 0) and np.all(x <= 1.05)
    assert np.allclose(x[:, 3], x[0, 3]) and np.allclose(x[:, 8], 0.25)


def test_training_learns_a_crossover():
    # synthetic cost table: push costs grow with the frontier, pull costs
    # with the unfinished edges; the fitted model must pick the cheaper side
    rng = np.random.default_rng(1)
    k = 600
    nf = 10 ** rng.uniform(0, 6, k)
    mf = nf * 16
    mu = 10 ** rng.uniform(3, 8, k)
    x = S.features(1 << 22, 1.28e8, nf, mf, mu, rng.integers(2, 12, k), nf / 4, 64)
    y = np.stack([np.log2(mf / 200 + 5), np.log2(mu / 800 + 5), np.log2(mf / 150 + 30)], 1).astype(np.float32)
    y[::3, 2] = np.nan  # rows without a dense measurement
    p, loss = S.train(x, y, epochs=1500, log=None)
    assert loss < 0.1
    w = S.flatten(p)
    choice = S.pick(w, x, (S.PUSH, S.PULL))
    truth = np.where(y[:, 0] < y[:, 1], S.PUSH, S.PULL)
    clear = np.abs(y[:, 0] - y[:, 1]) > 0.5
    assert np.mean(choice[clear] == truth[clear]) > 0.95
