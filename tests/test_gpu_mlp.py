"""The learned warm start on the GPU.

* The network's tensor-core kernels (tcgen05 GEMMs with fused epilogues)
  against the CPU oracle (oracle/mlp_oracle.py, same bf16 rounding points):
  loss and every weight/bias gradient, predictions, and one Adam step.
  Tolerances: relative 5e-3 in norm for gradients and 2e-3 for predictions.
  The only differences are fp32 accumulation order and the bf16 values that
  this order pushes across a rounding boundary (0.4 % each); they compound
  through the layers, measured 1e-7 at width 128 and 2.3e-3 for the first
  layer of the 5664 -> 3 x 512 -> 3776 network.  An error in a tile, a tail
  or an epilogue is of order 1.  Adam: 1e-5 absolute per parameter for a step
  of lr 1e-3 wherever the gradient's sign is stable.
* Training on the GPU reduces the loss.
* What the trained network gains: batched Newton from the predicted start
  needs fewer iterations than from the flat start, on held-out scenarios,
  and converges to the same solution (|V|, theta within 1e-6).
* Instances of a warm-started launch that run from their own start (chosen
  up front, or after a failed predicted run, restarted in the same launch)
  match the flat-start solve bit for bit, non-converging ones included."""
import numpy as np
import pytest

import mlp_oracle as mo

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(1e-30, np.linalg.norm(b)))


@pytest.mark.parametrize("n_in,n_out,width,n,skip", [(40, 36, 128, 64, False), (40, 36, 128, 64, True),
                                                     (300, 200, 256, 136, True), (5664, 3776, 512, 256, True)])
def test_gradients_match_oracle(gb, n_in, n_out, width, n, skip):
    m = gb.MLP(n_in, n_out, width=width, n_layers=3, skip=skip, seed=11)
    rng = np.random.default_rng(n_in)
    Xn = rng.normal(size=(n, n_in)).astype(np.float32)
    Yn = rng.normal(size=(n, n_out)).astype(np.float32)
    params = m.params()
    # non-zero biases and skip so that those paths are exercised
    params = [(W, (0.05 * rng.normal(size=b.shape)).astype(np.float32)) if b is not None else
              ((0.3 / np.sqrt(n_in) * rng.normal(size=W.shape)).astype(np.float32), None) for W, b in params]
    m.set_params(params)
    loss, grads = m.gradients(Xn, Yn)
    lo, go = mo.loss_and_grads(params, Xn, Yn, emulate=True)
    assert abs(loss - lo) <= 1e-4 * lo
    assert len(grads) == len(go) == 4 + skip
    for l, ((gw, gbias), (ow, ob)) in enumerate(zip(grads, go)):
        assert gw.shape == ow.shape
        assert rel(gw, ow) < 5e-3, f"layer {l} dW"
        if ob is not None:
            assert rel(gbias, ob) < 5e-3, f"layer {l} db"


def test_metric_loss_gradients_match_oracle(gb):
    n_in, n_out, n = 300, 200, 128
    m = gb.MLP(n_in, n_out, width=256, n_layers=3, seed=12)
    rng = np.random.default_rng(12)
    Xn = rng.normal(size=(n, n_in)).astype(np.float32)
    Yn = rng.normal(size=(n, n_out)).astype(np.float32)
    A = (rng.normal(size=(n_out, 150)) / np.sqrt(n_out)).astype(np.float32)
    m.set_loss_metric(A, 0.01)
    params = m.params()
    params[-1] = ((0.3 / np.sqrt(n_in) * rng.normal(size=params[-1][0].shape)).astype(np.float32), None)
    m.set_params(params)
    loss, grads = m.gradients(Xn, Yn)
    lo, go = mo.loss_and_grads(params, Xn, Yn, emulate=True, metric=(A, 0.01))
    assert abs(loss - lo) <= 2e-3 * lo
    for l, ((gw, gbias), (ow, ob)) in enumerate(zip(grads, go)):
        assert rel(gw, ow) < 5e-3, f"layer {l} dW"
        if ob is not None:
            assert rel(gbias, ob) < 5e-3, f"layer {l} db"


def _normalise(m, X, Y):
    nm = m.norm()
    Xn = (X.astype(np.float32) - nm["in_mean"]) * nm["in_scale"]
    Yn = (Y.astype(np.float32) - nm["out_mean"]) / nm["out_scale"]
    return Xn, Yn, nm


def test_predict_matches_oracle(gb):
    rng = np.random.default_rng(2)
    m = gb.MLP(300, 200, width=256, n_layers=3, seed=2)
    X = rng.normal(2.0, 3.0, (333, 300)).astype(np.float32)
    Y = rng.normal(-1.0, 0.5, (333, 200)).astype(np.float32)
    m.set_data(X, Y)
    Xn, _, nm = _normalise(m, X, Y)
    params = m.params()
    params[-1] = ((0.05 * rng.normal(size=params[-1][0].shape)).astype(np.float32), None)
    m.set_params(params)
    P = m.predict(X)
    y, _ = mo.forward(params, Xn, emulate=True)
    ref = y * nm["out_scale"] + nm["out_mean"]
    assert P.shape == ref.shape
    assert rel(P - nm["out_mean"], ref - nm["out_mean"]) < 2e-3


def test_one_training_step_matches_oracle_adam(gb):
    rng = np.random.default_rng(3)
    B = 64
    m = gb.MLP(40, 36, width=128, n_layers=3, seed=3)
    X = rng.normal(size=(B, 40)).astype(np.float32)
    Y = rng.normal(size=(B, 36)).astype(np.float32)
    m.set_data(X, Y)
    Xn, Yn, _ = _normalise(m, X, Y)
    p0 = m.params()
    loss, _ = m.train(1, batch=B, lr=1e-3, seed=1)
    p1 = m.params()
    lo, g = mo.loss_and_grads(p0, Xn, Yn, emulate=True)
    assert abs(loss[0] - lo) <= 1e-4 * lo
    z = lambda x: None if x is None else np.zeros_like(x, dtype=np.float64)
    state = [(z(W), z(W), z(b), z(b)) for W, b in p0]
    f64 = lambda x: None if x is None else x.astype(np.float64)
    want, _ = mo.adam_step([(f64(W), f64(b)) for W, b in p0], g, state, t=1, lr=1e-3)
    assert len(p1) == 5
    for (W0, b0), (W1, b1), (Ww, bw), (gW, gbias) in zip(p0, p1, want, g):
        for a0, a1, aw, ga in ((W0, W1, Ww, gW), (b0, b1, bw, gbias)):
            if a0 is None:
                continue
            stable = np.abs(ga) > 1e-2 * np.max(np.abs(ga))
            assert np.max(np.abs((a1 - a0) - (aw - a0))[stable]) < 1e-5
            # where the gradient is ~0 the first Adam step is +-lr or 0: bounded by lr
            assert np.max(np.abs(a1 - a0)) <= 1e-3 * (1 + 1e-3)


def test_training_reduces_loss(gb):
    rng = np.random.default_rng(4)
    n = 4096
    X = rng.normal(size=(n, 64)).astype(np.float32)
    A = rng.normal(size=(64, 48)) / 8
    Y = (np.tanh(X @ A) + 0.1 * (X[:, :48] ** 2)).astype(np.float32)
    m = gb.MLP(64, 48, width=256, n_layers=3, seed=4)
    m.set_data(X, Y)
    loss, ms = m.train(15, batch=256, lr=1e-3, seed=4)
    assert np.all(np.isfinite(loss))
    assert loss[-1] < 0.2 * loss[0]
    assert ms > 0


def _scenarios(base, n, rng):
    lf = rng.uniform(0.7, 1.3, (n, len(base["Pload"])))
    gf = rng.uniform(0.85, 1.15, (n, len(base["Pg"])))
    return base["Pload"] * lf, base["Qload"] * lf, base["Pg"] * gf


@pytest.fixture(scope="module")
def warm_net(gb):
    """A 118-bus grid and a network trained on 4,096 of its solved load
    scenarios (loss: the squared linearised mismatch of the predicted start
    plus 1 % MSE)."""
    grid = gb.generate(2, 20261205)
    base = grid.buses()
    nB = grid.nB
    rng = np.random.default_rng(5)
    solver = gb.Batch([grid], precision=gb.PREC_FP64, tolerancia=1e-8, no_max_iter=30, lim_inj_reat=0)
    Pl, Ql, Pg = _scenarios(base, 4096, rng)
    solver.set_instances(np.zeros(len(Pl), np.int32), Pload=Pl.ravel(), Qload=Ql.ravel(), Pg=Pg.ravel())
    solver.solve()
    r = solver.results()
    solver.close()
    ok = r["status"] == 0
    assert ok.mean() > 0.95
    V, th = r["V"].reshape(-1, nB)[ok], r["theta"].reshape(-1, nB)[ok]
    X = gb.warm_features(Pg[ok] - Pl[ok], base["Qg"] - Ql[ok], np.tile(base["V0"], (ok.sum(), 1)))
    Y = np.concatenate([V, th], axis=1)
    m = gb.MLP(3 * nB, 2 * nB, width=256, n_layers=3, seed=5)
    m.set_data(X, Y)
    plain = gb.Solver(grid, tolerancia=1e-8, no_max_iter=30, lim_inj_reat=0)
    M = gb.warm_loss_metric(plain, V.mean(0), th.mean(0), m.norm()["out_scale"])
    m.set_loss_metric(M, 0.01)
    loss, _ = m.train(40, batch=128, lr=1e-3, lr_final=1e-5, seed=5)
    return grid, m, loss


def test_warm_start_saves_iterations(gb, warm_net):
    grid, m, loss = warm_net
    base = grid.buses()
    nB = grid.nB
    rng = np.random.default_rng(55)
    solver = gb.Batch([grid], precision=gb.PREC_FP64, tolerancia=1e-8, no_max_iter=30, lim_inj_reat=0)

    def solve(Pl, Ql, Pg):
        n = len(Pl)
        solver.set_instances(np.zeros(n, np.int32), Pload=Pl.ravel(), Qload=Ql.ravel(), Pg=Pg.ravel())
        solver.solve()
        return solver.results()

    assert loss[-1] < 0.05 * loss[0]
    # held-out scenarios: flat start, then the learned start
    Pl, Ql, Pg = _scenarios(base, 512, rng)
    flat = solve(Pl, Ql, Pg)
    w = solver.solve_warm(m)
    warm = solver.results()
    both = (flat["status"] == 0)
    assert both.mean() > 0.95
    assert np.all(warm["status"][both] == 0)
    assert np.all(warm["final_mismatch"][both] <= 1e-8)
    sel = np.repeat(both, nB)
    assert np.max(np.abs(warm["V"][sel] - flat["V"][sel])) <= 1e-6
    assert np.max(np.abs(warm["theta"][sel] - flat["theta"][sel])) <= 1e-6
    kind = w["start_kind"]
    assert (kind == 2).mean() < 0.05
    assert (kind >= 1).mean() > 0.9
    it_flat = flat["iterations"][both].mean()
    it_warm = (warm["iterations"] + np.where(kind == 2, w["warm_iterations"], 0))[both].mean()
    assert it_warm < it_flat - 0.5, (it_warm, it_flat)


def test_warm_start_without_v0_features(gb):
    """A network over [Pliq | Qliq] alone (2 nB inputs, for scenario sets whose
    starting voltages do not vary): the batch builds those features itself,
    the predicted start is taken for most scenarios, and every answer equals
    the flat-start solve's within 1e-6 with fewer iterations (a smaller
    network than the 1,888-bus benchmark's, 40 epochs: 4.0 -> ~3.7)."""
    grid = gb.generate(2, 20261205)
    base = grid.buses()
    nB = grid.nB
    rng = np.random.default_rng(7)
    solver = gb.Batch([grid], precision=gb.PREC_FP64, tolerancia=1e-8, no_max_iter=30, lim_inj_reat=0)

    def solve(Pl, Ql, Pg):
        solver.set_instances(np.zeros(len(Pl), np.int32), Pload=Pl.ravel(), Qload=Ql.ravel(), Pg=Pg.ravel())
        solver.solve()
        return solver.results()

    Pl, Ql, Pg = _scenarios(base, 4096, rng)
    r = solve(Pl, Ql, Pg)
    ok = r["status"] == 0
    V, th = r["V"].reshape(-1, nB)[ok], r["theta"].reshape(-1, nB)[ok]
    X = gb.warm_features(Pg[ok] - Pl[ok], base["Qg"] - Ql[ok])
    assert X.shape[1] == 2 * nB
    m = gb.MLP(2 * nB, 2 * nB, width=256, n_layers=3, seed=7)
    m.set_data(X, np.concatenate([V, th], axis=1))
    plain = gb.Solver(grid, tolerancia=1e-8, no_max_iter=30, lim_inj_reat=0)
    m.set_loss_metric(gb.warm_loss_metric(plain, V.mean(0), th.mean(0), m.norm()["out_scale"]), 0.01)
    loss, _ = m.train(40, batch=128, lr=1e-3, lr_final=1e-5, seed=7)
    assert loss[-1] < 0.05 * loss[0]
    Pl, Ql, Pg = _scenarios(base, 256, rng)
    flat = solve(Pl, Ql, Pg)
    w = solver.solve_warm(m)
    warm = solver.results()
    both = flat["status"] == 0
    assert np.all(warm["status"][both] == 0)
    sel = np.repeat(both, nB)
    assert np.max(np.abs(warm["V"][sel] - flat["V"][sel])) <= 1e-6
    assert np.max(np.abs(warm["theta"][sel] - flat["theta"][sel])) <= 1e-6
    kind = w["start_kind"]
    assert (kind >= 1).mean() > 0.9
    it_warm = (warm["iterations"] + np.where(kind == 2, w["warm_iterations"], 0))[both].mean()
    assert it_warm < flat["iterations"][both].mean() - 0.25


def test_warm_start_iteration0_is_a_chord_step_at_the_mean_output(gb):
    """Iteration 0 of a predicted run factors no Jacobian of its own: it solves
    with the shared factor of the Jacobian at the network's mean output.  With
    every weight zero the network predicts that mean for every scenario, so
    the chord step is the Newton step from the predicted start: iterations,
    status, |V| and theta equal those of a plain solve started from the same
    state (the two factors differ in rounding only)."""
    grid = gb.generate(2, 20261205)
    base = grid.buses()
    nB, n = grid.nB, 256
    rng = np.random.default_rng(11)
    b = gb.Batch([grid], precision=gb.PREC_FP64, tolerancia=1e-8, no_max_iter=30, lim_inj_reat=0)
    Pl, Ql, Pg = _scenarios(base, n, rng)
    gi = np.zeros(n, np.int32)
    b.set_instances(gi, Pload=Pl.ravel(), Qload=Ql.ravel(), Pg=Pg.ravel())
    b.solve()
    r = b.results()
    ok = r["status"] == 0
    assert ok.mean() > 0.95
    mV = r["V"].reshape(-1, nB)[ok].mean(0).astype(np.float32)
    mt = r["theta"].reshape(-1, nB)[ok].mean(0).astype(np.float32)
    m = gb.MLP(3 * nB, 2 * nB, width=64, n_layers=2, seed=1)
    m.set_norm(np.zeros(3 * nB, np.float32), np.ones(3 * nB, np.float32), np.concatenate([mV, mt]),
               np.ones(2 * nB, np.float32))
    m.set_params([(np.zeros_like(W), None if c is None else np.zeros_like(c)) for W, c in m.params()])
    w = b.solve_warm(m)
    warm = b.results()
    kind = w["start_kind"]
    t = base["type"]
    V0 = np.where(t >= 2, base["V0"], mV.astype(np.float64))
    th0 = np.where(t == 3, base["theta0"], mt.astype(np.float64))
    b.set_instances(gi, Pload=Pl.ravel(), Qload=Ql.ravel(), Pg=Pg.ravel(), V0=np.tile(V0, n), theta0=np.tile(th0, n))
    b.solve()
    plain = b.results()
    b.close()
    sel = kind == 1
    assert sel.mean() > 0.9
    assert np.array_equal(warm["iterations"][sel], plain["iterations"][sel])
    assert np.array_equal(warm["status"][sel], plain["status"][sel])
    rows = np.repeat(sel, nB)
    assert np.max(np.abs(warm["V"][rows] - plain["V"][rows])) <= 1e-10
    assert np.max(np.abs(warm["theta"][rows] - plain["theta"][rows])) <= 1e-10


@pytest.mark.parametrize("prec", ["PREC_FP64", "PREC_FP32_IR"])
def test_warm_start_own_start_runs_match_flat_start(gb, warm_net, prec):
    """Instances that run from their own start in a warm-started launch -- the
    ones whose prediction was not chosen (start kind 0) and the ones whose
    predicted run failed and started again in the same launch (kind 2) -- give
    exactly what the flat-start solve gives: iterations (no_max_iter for the
    non-converging), status, switch events, |V| and theta bit for bit.  The
    network is the one of test_warm_start_saves_iterations; reactive limits
    are on, and a fifth of the scenarios are loaded past the point where
    Newton converges."""
    grid, m, _ = warm_net
    base = grid.buses()
    nB = grid.nB
    rng = np.random.default_rng(6)
    opts = dict(tolerancia=1e-8, no_max_iter=30, lim_inj_reat=1)
    solver = gb.Batch([grid], precision=getattr(gb, prec), **opts)
    Pl, Ql, Pg = _scenarios(base, 256, rng)
    heavy = rng.uniform(1.8, 2.6, (64, nB))
    Pl = np.concatenate([Pl, base["Pload"] * heavy])
    Ql = np.concatenate([Ql, base["Qload"] * heavy])
    Pg = np.concatenate([Pg, np.tile(base["Pg"], (64, 1))])
    order = rng.permutation(len(Pl))
    Pl, Ql, Pg = Pl[order], Ql[order], Pg[order]
    n = len(Pl)
    solver.set_instances(np.zeros(n, np.int32), Pload=Pl.ravel(), Qload=Ql.ravel(), Pg=Pg.ravel())
    solver.solve()
    flat = solver.results()
    ev_flat = [solver.events(i) for i in range(n)]
    ok = flat["status"] == 0
    assert 0 < (~ok).sum() < n // 2
    w = solver.solve_warm(m)
    warm = solver.results()
    kind = w["start_kind"]
    own = kind != 1
    assert own.any() and (kind == 1).any()
    # some non-converging scenario ran from its own start for all no_max_iter iterations
    assert (own & ~ok).any()
    sel = np.repeat(own, nB)
    for k in ("iterations", "status", "n_events"):
        np.testing.assert_array_equal(warm[k][own], flat[k][own], err_msg=k)
    np.testing.assert_array_equal(warm["V"][sel], flat["V"][sel])
    np.testing.assert_array_equal(warm["theta"][sel], flat["theta"][sel])
    for i in np.flatnonzero(own):
        np.testing.assert_array_equal(solver.events(i), ev_flat[i])
    assert np.all(w["warm_iterations"][kind == 0] == 0)
    assert np.all((w["warm_iterations"][kind == 2] >= 1) & (w["warm_iterations"][kind == 2] <= 10))
    # the predicted runs that were kept converged; without limit switches on
    # either path, to the flat start's solution
    assert np.all(warm["status"][kind == 1] == 0)
    kept = (kind == 1) & ok & (flat["n_events"] == 0) & (warm["n_events"] == 0)
    assert kept.any()
    s1 = np.repeat(kept, nB)
    assert np.max(np.abs(warm["V"][s1] - flat["V"][s1])) <= 1e-6
    assert np.max(np.abs(warm["theta"][s1] - flat["theta"][s1])) <= 1e-6


def test_warm_start_in_flight_on_two_batches(gb, warm_net):
    """Two batches sharing one network, both warm-started solves launched
    before either is waited for (each batch has its own stream and network
    workspace): each gives what its synchronous solve_warm gives, also after
    the timed round-robin of gbpf_batch_time_warm_pipelined."""
    grid, m, _ = warm_net
    base = grid.buses()
    opts = dict(tolerancia=1e-8, no_max_iter=30, lim_inj_reat=0)
    rng = np.random.default_rng(77)
    sets = [_scenarios(base, n, rng) for n in (300, 517)]
    ref = []
    for Pl, Ql, Pg in sets:
        b = gb.Batch([grid], precision=gb.PREC_FP32_IR, **opts)
        b.set_instances(np.zeros(len(Pl), np.int32), Pload=Pl.ravel(), Qload=Ql.ravel(), Pg=Pg.ravel())
        w = b.solve_warm(m)
        ref.append((w, b.results()))
        b.close()
    bs = []
    for Pl, Ql, Pg in sets:
        b = gb.Batch([grid], precision=gb.PREC_FP32_IR, **opts)
        b.set_instances(np.zeros(len(Pl), np.int32), Pload=Pl.ravel(), Qload=Ql.ravel(), Pg=Pg.ravel())
        b.solve_warm_launch(m)
        bs.append(b)
    with pytest.raises(gb.GbpfError):
        bs[0].set_instances(np.zeros(len(sets[0][0]), np.int32))  # refused while in flight
    for b, (w0, r0) in zip(bs, ref):
        w = b.solve_warm_wait()
        r = b.results()
        np.testing.assert_array_equal(w["start_kind"], w0["start_kind"])
        np.testing.assert_array_equal(w["warm_iterations"], w0["warm_iterations"])
        for k in ("iterations", "status", "V", "theta"):
            np.testing.assert_array_equal(r[k], r0[k], err_msg=k)
        with pytest.raises(gb.GbpfError):
            b.solve_warm_wait()  # nothing in flight
    # timed round-robin over both batches: every step a full warm-started
    # solve, the results of each batch's last step those of its own solve
    assert gb.time_warm_pipelined(bs, m, 5) > 0
    for b, (w0, r0) in zip(bs, ref):
        np.testing.assert_array_equal(b.results()["V"], r0["V"])
    # chained on the device (gbpf_batch_follow): the second starts when the
    # first has ended, the host enqueues both before waiting; same answers
    bs[0].solve_warm_launch(m)
    bs[1].follow(bs[0])
    bs[1].solve_warm_launch(m)
    for b, (w0, r0) in zip(bs, ref):
        w = b.solve_warm_wait()
        np.testing.assert_array_equal(w["start_kind"], w0["start_kind"])
        np.testing.assert_array_equal(b.results()["theta"], r0["theta"])


def test_gemm_wait_limit_runs_out_and_the_handle_recovers(gb):
    """A GEMM whose operand-ring waits may last 1 clock cycle cannot wait for
    its first TMA tile (hundreds of cycles away): every such wait runs out, the
    CTA drains its copies and tensor-core work, frees its tensor memory and
    returns, and the call reports GBPF_E_TIMEOUT.  With the default limit the
    same handle predicts again, bit for bit what it predicted before."""
    m = gb.MLP(1024, 256, width=256, n_layers=2, skip=True, seed=21)
    X = np.random.default_rng(21).normal(size=(512, 1024)).astype(np.float32)
    before = m.predict(X)
    m.set_wait_limit(1)
    with pytest.raises(gb.GbpfError) as e:
        m.predict(X)
    assert e.value.status == gb.E_TIMEOUT
    assert "wait ran out" in str(e.value)
    m.set_wait_limit(0)
    np.testing.assert_array_equal(m.predict(X), before)
