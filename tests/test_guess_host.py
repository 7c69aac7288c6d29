"""Host logic of the learned guess corrector without a GPU: its features,
the amplitude scales, the held-out split and the gate that enables the
correction only when it beats the plain guess on held-out steps."""
from types import SimpleNamespace

import numpy as np
import pytest

from hofstadter_hubbard_tsc_gb300.guess import NFEAT, LearnedGuess, _lw


class StubNet:
    """forward returns the stored target of a recorded feature matrix (or 0)."""

    def __init__(self, exact):
        self.exact, self.table = exact, {}

    def forward(self, X):
        return self.table.get(X.tobytes(), np.zeros(len(X))) if self.exact else np.zeros(len(X))

    def train(self, X, T, W=None, epochs=0, lr=0.0):
        return 0.0

    def free(self):
        pass


def _subs(n):
    return [SimpleNamespace(sys_num_up=4 + k % 3, sys_num_down=k % 2, env_num_up=10 - k % 3, env_num_down=k % 2,
                            sys_dim=8 + k, env_dim=9 + k) for k in range(n)]


def test_features_and_previous_weights():
    g = LearnedGuess(None, 16, 14, mlp=StubNet(False))
    subs = _subs(5)
    wg = np.array([0.5, 0.2, 0.2, 0.1, 0.0])
    X = g.features((6, 8), subs, wg)
    assert X.shape == (5, NFEAT)
    np.testing.assert_allclose(X[:, 0], _lw(wg))
    np.testing.assert_allclose(X[:, 1], X[:, 0])
    assert not X[:, 2].any()
    np.testing.assert_allclose(X[:, 3], [s.sys_num_up / 14 for s in subs])
    np.testing.assert_allclose(X[:, 8], 6 / 16)
    g.prev[(6, 8)] = {(s.sys_num_up, s.sys_num_down, s.env_num_up, s.env_num_down): 0.3 for s in subs[:2]}
    X2 = g.features((6, 8), subs, wg)
    np.testing.assert_allclose(X2[:2, 1], _lw(np.array([0.3, 0.3])))
    np.testing.assert_allclose(X2[:, 2], [1, 1, 0, 0, 0])


def test_scales_are_clipped_and_skip_empty_sectors():
    s = LearnedGuess.scales(np.array([0.0, 1.0, -1.0, 2 * np.log10(1.5) / 14, 1.0]),
                            np.array([0.1, 0.1, 0.1, 0.1, 1e-9]))
    np.testing.assert_allclose(s, [1.0, 2.0, 0.5, 1.5, 1.0])


@pytest.mark.parametrize("exact", [True, False])
def test_gate_opens_only_when_the_network_beats_the_plain_guess(exact):
    net = StubNet(exact)
    g = LearnedGuess(None, 16, 14, mlp=net, min_samples=4)
    rng = np.random.default_rng(2)
    subs = _subs(6)
    for step in range(10):
        wg = rng.uniform(0.05, 1.0, 6)
        wg /= wg.sum()
        wc = wg * rng.uniform(0.4, 2.5, 6)
        wc /= wc.sum()
        X = g.features((step + 2, 12 - step), subs, wg)
        T = _lw(wc) - X[:, 0]
        net.table[X.tobytes()] = T
        g.X.append(X)
        g.T.append(T)
        g.W.append(np.maximum(wc, wg) + 1e-8)
        g.WG.append(wg)
        g.WC.append(wc)
    assert len(g.data(held_out=True)[1]) == 2 * 6 and len(g.data(held_out=False)[1]) == 8 * 6
    assert g.train() == 0.0
    h_net, h_plain = g.val
    assert h_plain > 0
    if exact:
        assert h_net < 1e-20 and g.enabled
    else:
        assert h_net == pytest.approx(h_plain) and not g.enabled
