"""The learned proposal gate on the GPU, through the C ABI.

* The trainer's forward pass, loss gradient and Adam step against the float64 oracle
  (``oracle/prop_oracle.py``): logits within 1e-4 of their largest magnitude, each layer's
  gradient within 1e-4 of its largest magnitude (FP32 accumulation over up to 10^5 terms), the
  Adam update within 1e-5 relative.
* Training is deterministic (per-example partial gradients summed in example order).
* A gate with every cell open leaves the sorter's spikes bit for bit unchanged; with a gate set,
  every spike lies in a cell the oracle (BF16 weights, FP32 biases) opens.
* Trained on the plain matcher's labels of a 384-channel / 500-template recording, the gate keeps
  the plain matcher's spikes (recall) on held-out seeds at 5 and 40 Hz while closing most cells.
"""
import numpy as np
import pytest

from livespikesorter_gb300 import proposal, sorter, synth
from oracle import prop_oracle as po

from lss_testutil import match_spikes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

W_S, NT_S, C_S = 200, 20, 40


def _test_params(seed):
    """init_params with a livelier output layer, so the logits vary across samples."""
    rng = np.random.default_rng(seed)
    p = proposal.init_params(seed)
    wo, bo = po.offsets()[3]
    p[wo:bo] = rng.normal(0.0, 0.2, bo - wo).astype(np.float32)
    return p


def _bf16_weights(p):
    """The gate's device copy: weights rounded to BF16 (nearest even), biases kept in FP32."""
    q = np.array(p, np.float32)
    for wo, bo in po.offsets():
        u = q[wo:bo].view(np.uint32).astype(np.uint64)
        r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
        q[wo:bo] = r.view(np.float32)
    return q


@pytest.fixture(scope="module")
def small():
    rng = np.random.default_rng(7)
    Z = rng.normal(0.0, 1.0, (3, W_S, C_S)).astype(np.float32)
    pairs = proposal.all_pairs(3, proposal.neighbourhoods(C_S))
    lab = (rng.random((len(pairs), proposal.n_windows(W_S, NT_S))) < 0.3).astype(np.uint8)
    return Z, torch.from_numpy(Z).cuda(), pairs, lab


def test_forward_matches_oracle(small):
    Z, z, pairs, _ = small
    p = _test_params(2)
    with proposal.ProposalTrainer(W_S, NT_S, max_examples=16, params=p) as tr:
        lg, zw = tr.forward(z, pairs)
    _, ref = po.forward(p, po.gather_examples(Z, pairs))
    scale = np.abs(ref).max()
    assert np.abs(lg - ref).max() <= 1e-4 * scale
    zr, _ = po.window_max(ref, W_S, NT_S)
    assert np.abs(zw - zr).max() <= 1e-4 * scale


@pytest.mark.parametrize("C,W,nt", [(8, 97, 10), (16, 300, 61), (23, 1622, 61)])
def test_forward_ragged_shapes(C, W, nt):
    """Probes narrower than a neighbourhood (zero-padded channels), a last window shorter than 32
    samples, a neighbourhood start that is not a multiple of 8."""
    rng = np.random.default_rng(C)
    Z = rng.normal(0.0, 1.0, (2, W, C)).astype(np.float32)
    pairs = proposal.all_pairs(2, proposal.neighbourhoods(C))
    p = _test_params(9)
    with proposal.ProposalTrainer(W, nt, max_examples=len(pairs), params=p) as tr:
        lg, zw = tr.forward(torch.from_numpy(Z).cuda(), pairs)
    _, ref = po.forward(p, po.gather_examples(Z, pairs))
    assert np.abs(lg - ref).max() <= 1e-4 * np.abs(ref).max()
    zr, _ = po.window_max(ref, W, nt)
    assert zw.shape == zr.shape and np.abs(zw - zr).max() <= 1e-4 * np.abs(ref).max()


def test_trainer_rejects_bad_examples(small):
    _, z, pairs, lab = small
    with proposal.ProposalTrainer(W_S, NT_S, max_examples=4, params=_test_params(2)) as tr:
        with pytest.raises(sorter.SorterError):
            tr.forward(z, pairs[:5])                      # more than max_examples
        bad = pairs[:2].copy()
        bad[0, 0] = 3                                     # window past the 3 given
        with pytest.raises(sorter.SorterError):
            tr.forward(z, bad)
        bad = pairs[:2].copy()
        bad[1, 1] = C_S - 8                               # neighbourhood past the last channel
        with pytest.raises(sorter.SorterError):
            tr.step(z, bad, lab[:2])
        lg, _ = tr.forward(z, pairs[:4])                  # the handle still works
        assert np.isfinite(lg).all()


def test_gradient_matches_oracle(small):
    Z, z, pairs, lab = small
    p = _test_params(3)
    with proposal.ProposalTrainer(W_S, NT_S, max_examples=16, params=p) as tr:
        lg, _ = tr.forward(z, pairs)
        loss, g = tr.loss_grad(z, pairs, lab)
    # each window's maximum at the sample the device picked
    nw = proposal.n_windows(W_S, NT_S)
    arg = np.stack([NT_S + 32 * w + lg[:, NT_S + 32 * w:min(NT_S + 32 * (w + 1), W_S - NT_S)].argmax(1)
                    for w in range(nw)], 1)
    ref_loss, ref_g = po.loss_and_grad(p, po.gather_examples(Z, pairs), lab, W_S, NT_S, argmax=arg)
    assert loss == pytest.approx(ref_loss, rel=1e-5)
    for li, (wo, bo) in enumerate(po.offsets()):
        end = po.offsets()[li + 1][0] if li < 3 else po.param_count()
        for lo, hi in ((wo, bo), (bo, end)):
            scale = np.abs(ref_g[lo:hi]).max()
            assert np.abs(g[lo:hi] - ref_g[lo:hi]).max() <= 1e-4 * scale + 1e-12, (li, lo)


def test_adam_step_matches_oracle(small):
    _, z, pairs, lab = small
    p = _test_params(4)
    with proposal.ProposalTrainer(W_S, NT_S, max_examples=16, params=p, lr=1e-3) as tr:
        _, g = tr.loss_grad(z, pairs, lab)
        tr.step(z, pairs, lab)
        p1 = tr.params
    zero = np.zeros_like(p)
    ref, _, _ = po.adam_step(p, zero, zero, g, 1, lr=1e-3)
    np.testing.assert_allclose(p1, ref, rtol=1e-5, atol=1e-8)


def test_training_is_deterministic(small):
    _, z, pairs, lab = small
    out = []
    for _ in range(2):
        with proposal.ProposalTrainer(W_S, NT_S, max_examples=16, params=_test_params(5)) as tr:
            losses = [tr.step(z, pairs[i::2], lab[i::2]) for i in (0, 1, 0, 1)]
            out.append((losses, tr.params))
    assert out[0][0] == out[1][0]
    np.testing.assert_array_equal(out[0][1], out[1][1])
    assert out[0][0][2] < out[0][0][0]   # the loss of the same examples went down


@pytest.fixture(scope="module")
def gate_data(tmp_path_factory):
    cfg = synth.SynthConfig(n_chan=64, n_units=48, n_samples=8 * 1500 + 300, whiten_batch=3000, whiten_batches=2,
                            seed=31)
    rec = synth.make_recording(cfg)
    oss = synth.build_oss_input(rec)
    d = synth.write_oss_input(oss, tmp_path_factory.mktemp("prop") / "oss_input")
    wins = proposal.batch_windows(rec.data, 0, 6, 1500, 61)
    return d, wins, oss, rec.data


def _same_spikes(a, b):
    for x, y in zip(a, b):
        for f in ("time", "tmpl", "amp", "cluster"):
            np.testing.assert_array_equal(x[f], y[f])


def test_gate_with_every_cell_open_is_the_plain_sorter(gate_data):
    d, wins, _, _ = gate_data
    with sorter.OnlineSorter(d, batch_samples=1500, max_iters=50, group_batches=4) as s:
        plain = s.sort_windows(wins)
        s.set_proposal(_test_params(1), logit_threshold=-np.inf, dilate=0)
        gated = s.sort_windows(wins)
        cells, opened = s.proposal_stats()
        s.set_proposal(None)
        again = s.sort_windows(wins)
        assert s.proposal_stats() == (0, 0)
    assert sum(len(x) for x in plain) > 50
    _same_spikes(plain, gated)
    _same_spikes(plain, again)
    assert cells == opened == len(wins) * len(proposal.neighbourhoods(64)) * 47


def test_gate_on_the_streaming_path(gate_data):
    """The gate applies to pushed streams as well: all cells open gives the plain stream's spikes
    bit for bit; a gate with cells closed changes them and counts every batch's cells."""
    d, _, _, data = gate_data
    with sorter.OnlineSorter(d, batch_samples=1500, max_iters=50, group_batches=3) as s:
        plain = s.sort_stream(data, chunk=2000)
    with sorter.OnlineSorter(d, batch_samples=1500, max_iters=50, group_batches=3) as s:
        s.set_proposal(_test_params(1), logit_threshold=-np.inf, dilate=0)
        gated = s.sort_stream(data, chunk=2000)
        cells, opened = s.proposal_stats()
    _same_spikes([plain], [gated])
    n_full = len(data) // 1500 - 1                   # windows certainly launched at full length
    assert cells == opened and cells % len(proposal.neighbourhoods(64)) == 0
    assert cells >= n_full * len(proposal.neighbourhoods(64)) * 47
    with sorter.OnlineSorter(d, batch_samples=1500, max_iters=50, group_batches=3) as s:
        s.set_proposal(_test_params(1), logit_threshold=1e30, dilate=0)   # every cell closed
        none = s.sort_stream(data, chunk=2000)
        cells, opened = s.proposal_stats()
    assert opened == 0 and cells > 0
    # the cells cover every window's interior, and the loop never accepts outside it
    assert len(plain) > 50 and len(none) == 0


def test_gated_spikes_lie_in_open_cells(gate_data):
    d, wins, oss, _ = gate_data
    p = _test_params(6)
    starts = proposal.neighbourhoods(64)
    owner = po.template_owner(oss.Wall3)
    with sorter.OnlineSorter(d, batch_samples=1500, max_iters=50, group_batches=4) as s:
        W, nt, n0 = wins.shape[1], s.info.nt, s.info.nt0min
        Z = np.stack([s.debug_stage(w, sorter.STAGE_PREPROCESSED) for w in wins])
        _, lg = po.forward(_bf16_weights(p), po.gather_examples(Z, proposal.all_pairs(len(wins), starts)))
        z, _ = po.window_max(lg, W, nt)
        z = z.reshape(len(wins), len(starts), -1)
        thr = float(np.median(z))
        s.set_proposal(p, logit_threshold=thr, dilate=1)
        gated = s.sort_windows(wins)
        cells, opened = s.proposal_stats()
    zd = proposal.dilated_logits(z, 1)
    margin = 1e-3 * np.abs(z).max()
    for j, sp in enumerate(gated):
        smp = sp["time"] + nt // 2 - n0
        inner = (smp >= nt) & (smp < W - nt)
        cell = zd[j, owner[sp["tmpl"][inner]], (smp[inner] - nt) // 32]
        assert np.all(cell > thr - margin)
    ref_open = int((zd > thr).sum())
    assert cells == zd.size
    assert abs(opened - ref_open) <= max(3, 0.002 * cells), (opened, ref_open)
    assert 0.2 * cells < opened < 0.95 * cells


@pytest.fixture(scope="module")
def dense_probe(tmp_path_factory):
    """384 channels, 500 units at 10 Hz: 64 batch windows for training."""
    cfg = synth.SynthConfig(n_chan=384, n_units=500, n_samples=64 * 1500 + 300, drift_um=20.0, whiten_batch=3000,
                            whiten_batches=3, seed=41)
    rec = synth.make_recording(cfg)
    oss = synth.build_oss_input(rec)
    d = synth.write_oss_input(oss, tmp_path_factory.mktemp("prop384") / "oss_input")
    return d, rec, oss


def test_learned_gate_keeps_the_plain_matchers_spikes(dense_probe):
    d, rec, oss = dense_probe
    NT, nt = 1500, 61
    starts = proposal.neighbourhoods(384)
    owner = proposal.template_owner(oss.Wall3)
    with sorter.OnlineSorter(d, batch_samples=NT, max_iters=50, group_batches=8) as s:
        wins = proposal.batch_windows(rec.data, 0, 64, NT, nt)
        labels, _ = proposal.plain_labels(s, wins, owner, len(starts))
        z = proposal.whitened(s, wins)
        with proposal.ProposalTrainer(NT + 2 * nt, nt, max_examples=64, seed=0) as tr:
            losses = proposal.train(tr, z, labels, starts, steps=300, batch=64, seed=0)
            zw = proposal.window_logits(tr, z, starts)
            params = tr.params
        assert losses[-20:].mean() < 0.5 * losses[:20].mean(), (losses[:5], losses[-5:])
        # the logit threshold keeps 99.9 % of the training windows' labelled cells open: held-out
        # recall then clears the metric's 99.5 % (measured 99.9-100 % at 5-40 Hz)
        thr = proposal.choose_threshold(zw, labels, 1, 0.999)
        s.set_proposal(params, logit_threshold=thr, dilate=1)
        results = {}
        for rate, seed in ((5.0, 101), (40.0, 102)):
            held = synth.rerecord(rec, seed, rate_hz=rate, n_samples=16 * NT + 300)
            hw = proposal.batch_windows(held.data, 0, 16, NT, nt)
            c0, o0 = s.proposal_stats()
            gated = np.concatenate(s.sort_windows(hw))
            c1, o1 = s.proposal_stats()
            s.set_proposal(None)
            plain = np.concatenate(s.sort_windows(hw))
            s.set_proposal(params, logit_threshold=thr, dilate=1)
            ri, _ = match_spikes(plain["time"], plain["tmpl"], gated["time"], gated["tmpl"])
            results[rate] = (len(ri) / max(1, len(plain)), (o1 - o0) / (c1 - c0), len(plain), len(gated))
    # the gain: most cells closed at 5 Hz (measured 23 % open); at 40 Hz most cells hold a spike
    # and stay open
    for rate, (recall, open_frac, n_plain, n_gated) in results.items():
        assert n_plain > 200, results
        assert recall >= 0.995, results
        assert open_frac <= (0.4 if rate == 5.0 else 0.95), results
