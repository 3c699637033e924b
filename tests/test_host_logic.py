"""Host-side logic of the transient driver and the predictor that runs
without a GPU: the seeded tip load, the training pairs, the network's input
channels."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from igap4_gb300.predictor import Scales, features, make_samples  # noqa: E402
from igap4_gb300.transient import TipLoad  # noqa: E402


def test_tip_load_is_seeded_and_in_range():
    a, b = TipLoad(seed=7), TipLoad(seed=7)
    np.testing.assert_array_equal(a.amp, b.amp)
    np.testing.assert_array_equal(a.freq, b.freq)
    assert np.all((a.amp >= 0) & (a.amp <= 1e-3)) and np.all((a.freq >= 0.5) & (a.freq <= 5.0))
    t = 0.37
    expect = -np.sum(a.amp * np.sin(2 * np.pi * a.freq * t))
    assert a.value(t) == pytest.approx(expect, rel=0, abs=1e-18)
    tab = a.table(t)
    assert tab.shape == (36,) and tab[6 * 1 + 2] == a.value(t)  # face x = L, order 0, z component
    assert np.count_nonzero(tab) == (1 if a.value(t) != 0 else 0)
    assert not np.array_equal(TipLoad(seed=8).amp, a.amp)


def test_training_pairs_are_corrections_to_extrapolation():
    rng = np.random.default_rng(3)
    states = rng.standard_normal((6, 12))
    loads = rng.standard_normal(6)
    X, Y = make_samples(states, loads, None)
    assert len(X) == len(Y) == 4  # n = 1 .. N-2
    for k, (x, y) in enumerate(zip(X, Y)):
        n = k + 1
        np.testing.assert_array_equal(x[0], states[n])
        np.testing.assert_array_equal(x[1], states[n - 1])
        np.testing.assert_array_equal(x[2], [0.0, 0.0, loads[n + 1] - loads[n]])
        np.testing.assert_allclose(states[n] + (states[n] - states[n - 1]) + y, states[n + 1], rtol=0, atol=1e-14)


@pytest.mark.parametrize("mode", ["load", "residual"])
def test_feature_channels(mode):
    P = 5
    un = torch.arange(3 * P, dtype=torch.float64)
    unm1 = -un
    sc = Scales(u=2.0, load=4.0, out=1.0, mode=mode)
    third = np.array([0.0, 0.0, 8.0]) if mode == "load" else torch.full((3 * P,), 8.0, dtype=torch.float64)
    x = features(un, unm1, third, sc)
    assert x.shape == (P, 9) and x.dtype == torch.float32
    np.testing.assert_allclose(x[:, 0:3].numpy().ravel(), un.numpy() / 2.0)
    np.testing.assert_allclose(x[:, 3:6].numpy().ravel(), -un.numpy() / 2.0)
    expect = np.tile([0.0, 0.0, 2.0], (P, 1)) if mode == "load" else np.full((P, 3), 2.0)
    np.testing.assert_allclose(x[:, 6:9].numpy(), expect)


def test_feature_channels_relative():
    """Step-relative inputs: u_n / s_u, the last increment in units of its own
    largest component, the load increment / s_load."""
    P = 4
    un = torch.arange(3 * P, dtype=torch.float64) * 0.5
    unm1 = un - torch.linspace(-3.0, 1.5, 3 * P, dtype=torch.float64)
    sc = Scales(u=2.0, load=4.0, out=1.0, mode="relative")
    x = features(un, unm1, np.array([0.0, 0.0, 8.0]), sc)
    inc = (un - unm1).numpy()
    np.testing.assert_allclose(x[:, 0:3].numpy().ravel(), un.numpy() / 2.0)
    np.testing.assert_allclose(x[:, 3:6].numpy().ravel(), inc / np.abs(inc).max(), rtol=1e-6)
    assert np.abs(x[:, 3:6].numpy()).max() == pytest.approx(1.0)
    np.testing.assert_allclose(x[:, 6:9].numpy(), np.tile([0.0, 0.0, 2.0], (P, 1)))
