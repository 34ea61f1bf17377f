"""Learned-start network on the device (sk_gnn_*) against the CPU oracle
(oracle/gnn_oracle.py), its training, and the learned start inside the solver."""
import os

import numpy as np
import pytest

import gnn_oracle as go

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(os.path.dirname(HERE), "soverign-gpu-accelerator-_gb300", "weights",
                       "learned_start_family3.npy")


def graph(sk, m, n, d, seed):
    lp = sk.random_lp(m, n, d, seed)
    rp, ci, v = lp.csr()
    rng = np.random.default_rng(seed)
    t = (rng.normal(0, 1.5, n), rng.normal(0, 1.5, n), rng.normal(0, 1, m))
    return lp, rp, ci, v, t


@pytest.mark.parametrize("m,n,d,seed", [(40, 90, 0.08, 5), (300, 700, 0.015, 6)])
def test_forward_matches_oracle(gpu, m, n, d, seed):
    sk = gpu
    lp, rp, ci, v, _ = graph(sk, m, n, d, seed)
    p = go.glorot_params(seed)
    net = sk.Gnn(seed)
    net.set_params(p)
    np.testing.assert_array_equal(net.get_params(), p)
    bt = sk.GnnBatch.from_arrays(m, n, rp, ci, v, lp.b, lp.c)
    lx, ls, y = net.predict(bt)
    rx, rs, ry, _, _ = go.forward(p, m, n, rp, ci, v, lp.b, lp.c, bf16=True)
    for a, r in ((lx, rx), (ls, rs), (y, ry)):
        assert np.max(np.abs(a - r)) <= 1e-4 * (1.0 + np.max(np.abs(r)))   # FP32 accumulation vs FP64
    bt.close()
    net.close()


@pytest.mark.parametrize("m,n,d,seed", [(40, 90, 0.08, 7), (300, 700, 0.015, 8)])
def test_gradients_match_oracle(gpu, m, n, d, seed):
    sk = gpu
    lp, rp, ci, v, t = graph(sk, m, n, d, seed)
    p = go.glorot_params(seed)
    net = sk.Gnn(seed)
    net.set_params(p)
    bt = sk.GnnBatch.from_arrays(m, n, rp, ci, v, lp.b, lp.c, t)
    loss, g = net.loss_grad(bt)
    _, _, _, rloss, cache = go.forward(p, m, n, rp, ci, v, lp.b, lp.c, t, bf16=True)
    rg = go.backward(cache)
    assert abs(loss - rloss) <= 1e-5 * rloss
    assert np.linalg.norm(g - rg) <= 1e-3 * np.linalg.norm(rg)
    lay, _ = go.layout()
    for name, (o, s) in lay.items():             # every parameter block, not just the big ones
        k = int(np.prod(s))
        ref = rg[o:o + k]
        assert np.linalg.norm(g[o:o + k] - ref) <= 2e-3 * np.linalg.norm(rg) + 1e-3 * np.linalg.norm(ref), name
    bt.close()
    net.close()


def test_training_on_captured_iterates_reduces_loss(gpu):
    sk = gpu
    lps = [sk.generate(3, 300000 + k) for k in range(3)]
    s = sk.Solver(lps, precision=sk.PREC_FP64, start=sk.START_MEHROTRA)
    s.set_capture(1e-2)
    s.run()
    assert all(s.result(k, want_vectors=False)[0]["status"] == 0 for k in range(3))
    bt = sk.GnnBatch.from_solver(s)
    s.close()
    net = sk.Gnn(3)
    first = net.train_step(bt, 3e-3)
    for _ in range(150):
        last = net.train_step(bt, 3e-3)
    assert np.isfinite(last) and last < 0.5 * first
    bt.close()
    net.close()


def test_learned_start_keeps_the_answer(gpu, oracle):
    # The start changes the path, never the result: held-out family members solved
    # from the learned start agree with a tight (1e-11) plain FP64 solve to 1e-8 and
    # meet 1e-8 on the oracle's independent residual check.
    sk = gpu
    net = sk.Gnn(5)
    if os.path.exists(WEIGHTS):
        net.load(WEIGHTS)
    lps = [sk.generate(3, 200000 + k) for k in range(4)]
    s = sk.Solver(lps, precision=sk.PREC_MIXED, start=sk.START_LEARNED)
    s.set_gnn(net)
    s.run()
    for k, lp in enumerate(lps):
        info, x, y, z = s.result(k)
        assert info["status"] == 0
        ref, *_ = sk.solve(lp, precision=sk.PREC_FP64, tol=1e-11)
        assert abs(info["objective"] - ref["objective"]) / (1 + abs(ref["objective"])) <= 1e-8
        meas = oracle.kkt_measures(lp, x, y, z)
        assert meas["rel_pinf"] <= 1e-8 and meas["rel_dinf"] <= 1e-8 and meas["rel_gap"] <= 1e-8
    s.close()
    net.close()


def test_solver_rejects_learned_start_without_network(gpu):
    sk = gpu
    s = sk.Solver([sk.generate(3, 200000)], start=sk.START_LEARNED)
    with pytest.raises(RuntimeError, match="network"):
        s.run()
    s.close()


@pytest.mark.skipif(not os.path.exists(WEIGHTS), reason="trained weights not present")
def test_trained_network_cuts_iterations_on_heldout_seeds(gpu):
    # What the trained network gains: held-out members of the family (never seen in
    # training or in choosing the acceptance rule), each solved alone from Mehrotra's
    # start and from the learned start (which falls back to Mehrotra's per LP).
    sk = gpu
    net = sk.Gnn(1)
    net.load(WEIGHTS)
    its = {sk.START_MEHROTRA: 0, sk.START_LEARNED: 0}
    used = 0
    for k in range(12):
        lp = sk.generate(3, 200300 + k)
        for start in (sk.START_MEHROTRA, sk.START_LEARNED):
            s = sk.Solver([lp], precision=sk.PREC_MIXED, start=start)
            if start == sk.START_LEARNED:
                s.set_gnn(net)
            s.run()
            info = s.result(0, want_vectors=False)[0]
            assert info["status"] == 0
            its[start] += info["iterations"]
            if start == sk.START_LEARNED:
                used += info["learned_start"]
            s.close()
    print("iterations: mehrotra %d learned %d, learned start used on %d/12" %
          (its[sk.START_MEHROTRA], its[sk.START_LEARNED], used))
    assert used > 0
    assert its[sk.START_LEARNED] < its[sk.START_MEHROTRA]
