"""The proposal gate without a GPU: the oracle's gradient against central finite differences
(the oracle has no reference implementation to pin it, so this is its pin), and the host-side
pieces of the product (neighbourhoods, template owners through the C ABI, labels, threshold
choice, parameter layout) against the oracle."""
import numpy as np
import pytest

from livespikesorter_gb300 import proposal
from oracle import prop_oracle as po


def test_parameter_layout():
    assert po.param_count() == proposal.N_PARAMS == 65153
    p = proposal.init_params(3)
    assert p.dtype == np.float32 and p.shape == (proposal.N_PARAMS,)
    layers = po.unpack(p)
    assert [w.shape for w, _ in layers] == [(64, 16, 7), (64, 64, 7), (64, 64, 7), (1, 64, 7)]
    assert np.all(layers[0][1] == 0) and layers[3][1][0] == pytest.approx(np.log(0.1 / 0.9), rel=1e-6)


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = proposal.init_params(1).astype(np.float64)
    W, nt = 90, 12
    x = rng.normal(0.0, 1.0, (2, 16, W))
    lab = (rng.random((2, po.n_windows(W, nt))) < 0.4).astype(np.uint8)
    loss, g = po.loss_and_grad(p, x, lab, W, nt)
    assert np.isfinite(loss)
    # a sample of every layer's weights and biases, the output bias included
    idx = np.concatenate([rng.choice(off[1] - off[0], 6, replace=False) + off[0] for off in po.offsets()]
                         + [[o[1] for o in po.offsets()], [po.param_count() - 1]])
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (po.loss_and_grad(pp, x, lab, W, nt)[0] - po.loss_and_grad(pm, x, lab, W, nt)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * np.abs(g).max() + 1e-9, (i, fd, g[i])


def test_adam_oracle_first_step_moves_by_lr():
    p = np.ones(5, np.float32)
    g = np.array([1.0, -2.0, 0.5, 0.0, 3.0], np.float32)
    z = np.zeros(5, np.float32)
    p1, m, v = po.adam_step(p, z, z, g, 1, lr=1e-2)
    # first bias-corrected Adam step: -lr * sign(g) (to within eps)
    np.testing.assert_allclose(p1, p - 1e-2 * np.sign(g), atol=1e-6)


@pytest.mark.parametrize("C", [1, 8, 16, 17, 40, 100, 384])
def test_neighbourhoods_and_owners(C):
    starts = proposal.neighbourhoods(C)
    np.testing.assert_array_equal(starts, po.neighbourhood_starts(C))
    if C >= 16:
        assert starts[0] == 0 and starts[-1] == C - 16 and np.all(np.diff(starts) <= 8)
    rng = np.random.default_rng(C)
    Wall3 = rng.normal(0.0, 1.0, (30, 6, C)).astype(np.float32)
    np.testing.assert_array_equal(proposal.template_owner(Wall3), po.template_owner(Wall3))


def test_window_labels_match_oracle():
    rng = np.random.default_rng(5)
    W, nt, NB, T = 1622, 61, 47, 500
    owner = rng.integers(0, NB, T).astype(np.int32)
    s = rng.integers(0, W, 400)
    t = rng.integers(0, T, 400)
    np.testing.assert_array_equal(proposal.window_labels(s, t, owner, NB, W, nt),
                                  po.window_labels(s, t, owner, NB, W, nt))
    assert proposal.n_windows(W, nt) == po.n_windows(W, nt) == 47


@pytest.mark.parametrize("dilate", [0, 1, 2])
def test_threshold_choice_is_the_largest_that_keeps_recall(dilate):
    rng = np.random.default_rng(dilate)
    z = rng.normal(-3.0, 2.0, (20, 12, 47)).astype(np.float32)
    lab = (rng.random(z.shape) < 0.1).astype(np.uint8)
    z[lab > 0] += 3.0
    for target in (0.9, 0.99, 1.0):
        thr = proposal.choose_threshold(z, lab, dilate, target)
        opened = po.open_cells(z, thr, dilate)
        rec = (opened & (lab > 0)).sum() / (lab > 0).sum()
        assert rec >= target
        above = np.nextafter(np.float32(thr), np.float32(np.inf))
        above = np.nextafter(above, np.float32(np.inf))
        rec2 = (po.open_cells(z, above, dilate) & (lab > 0)).sum() / (lab > 0).sum()
        assert rec2 < target or rec2 == rec


def test_allowed_scores_follow_owner_cells():
    W, nt, NB = 200, 20, 3
    owner = np.array([0, 2, 1, 2], np.int32)
    mask = np.zeros((NB, po.n_windows(W, nt)), bool)
    mask[2, 1] = True
    a = po.allowed_scores(mask, owner, W, nt)
    assert a[:nt].all() and a[W - nt:].all()
    inner = a[nt:W - nt]
    rows = np.nonzero(inner[:, 1])[0]
    np.testing.assert_array_equal(rows, np.arange(32, 64))
    assert not inner[:, 0].any() and not inner[:, 2].any()
