"""Learned warm start: training kernels, tensor-core inference, and the
warm-started routing against the oracle.

- Gradients of the hand-written forward/backward kernels are checked against
  torch FP64 autograd of the same network and loss, and against central finite
  differences of the kernels' own loss.
- Inference (the tcgen05 GEMM: BF16 operands, FP32 accumulation in tensor
  memory) is checked against a torch emulation with the same BF16 roundings,
  and against the FP32 network.
- The routing kernel's warm-started solves are replayed by the oracle
  (oracle_mc_solve_warm) from the starting depths the kernel recorded: the
  whole discharge history is bit-identical, as are the iteration and fallback
  counts.
- The A/B test trains on pairs from plain runs of one network and routes a
  fresh-seed network with and without the model.
"""
import numpy as np
import pytest

import troute_gb300 as T
from oracle import troute_oracle as O
from troute_gb300 import synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TIGHT = (1e-8, 1e-10, 100, 5)
FLOOR = np.float32(1e-3)
NP = T.api.WARM_NPARAMS


def tight_cfg(**kw):
    return T.make_cfg(rtol=TIGHT[0], atol=TIGHT[1], maxiter=TIGHT[2], attempts=TIGHT[3], **kw)


def unpack(state):
    s = np.asarray(state, np.float64)
    o = 0
    W1 = s[o:o + 512].reshape(64, 8); o += 512
    b1 = s[o:o + 64]; o += 64
    W2 = s[o:o + 4096].reshape(64, 64); o += 4096
    b2 = s[o:o + 64]; o += 64
    w3 = s[o:o + 64]; o += 64
    b3 = s[o]; o += 1
    mu, sd = s[o:o + 8], s[o + 8:o + 16]
    mu_y, sd_y = s[o + 16], s[o + 17]
    return W1, b1, W2, b2, w3, b3, mu, sd, mu_y, sd_y


def features(pairs, mu, sd):
    """Standardised log features exactly as the kernels form them (float32)."""
    p = np.asarray(pairs, np.float32)
    raw = p[:, :8].copy()
    raw[:, :4] += FLOOR
    x = (np.log(raw) - np.float32(mu)[None, :].astype(np.float32)) / np.float32(sd)[None, :].astype(np.float32)
    return x.astype(np.float32)


def synthetic_pairs(n, seed):
    rng = np.random.default_rng(seed)
    q = np.exp(rng.normal(0.0, 1.5, (n, 4))).astype(np.float32)
    dx = rng.uniform(500, 5000, n)
    s0 = np.exp(rng.uniform(np.log(1e-5), np.log(1e-2), n))
    nn = rng.uniform(0.03, 0.08, n)
    bw = rng.uniform(2, 50, n)
    depth = 0.3 * (q[:, 1] + q[:, 3]) ** 0.6 * (nn / 0.05) ** 0.6 / (bw / 10) ** 0.5 / (s0 / 1e-3) ** 0.3
    return np.column_stack([q, dx, s0, nn, bw, depth]).astype(np.float32)


def random_state(pairs, seed):
    rng = np.random.default_rng(seed)
    st = np.zeros(T.api.WARM_NSTATE, np.float32)
    st[:NP] = rng.normal(0, 0.3, NP)
    raw = pairs[pairs[:, 8] > 0, :9].astype(np.float64)
    raw[:, :4] += 1e-3
    lg = np.log(raw)
    st[NP:NP + 8] = lg[:, :8].mean(0)
    st[NP + 8:NP + 16] = lg[:, :8].std(0)
    st[NP + 16] = lg[:, 8].mean()
    st[NP + 17] = lg[:, 8].std()
    return st


def torch_loss(state, pairs):
    """FP64 autograd reference of the training kernel's loss, mean (err^2)/2 over
    all rows (rows with a non-positive depth contribute no error)."""
    W1, b1, W2, b2, w3, b3, mu, sd, mu_y, sd_y = unpack(state)
    valid = pairs[:, 8] > 0
    x = torch.tensor(features(pairs, mu, sd).astype(np.float64))
    y = torch.tensor(((np.log(np.where(valid, pairs[:, 8], 1.0).astype(np.float32)) - np.float32(mu_y))
                      / np.float32(sd_y)).astype(np.float64))
    P = [torch.tensor(a, requires_grad=True) for a in (W1, b1, W2, b2, w3, np.array(b3))]
    silu = lambda z: z / (1 + torch.exp(-z))
    a1 = silu(x @ P[0].T + P[1])
    a2 = silu(a1 @ P[2].T + P[3])
    out = a2 @ P[4] + P[5]
    err = torch.where(torch.tensor(valid), out - y, torch.zeros_like(out))
    loss = 0.5 * (err ** 2).sum() / len(pairs)
    loss.backward()
    g = np.concatenate([p.grad.detach().numpy().ravel() for p in P])
    return float(loss.detach()), g


def test_gradients_match_torch_fp64():
    pairs = synthetic_pairs(300, 1)
    pairs[7, 8] = 0.0  # an invalid pair (no solve) adds no error
    st = random_state(pairs, 2)
    m = T.WarmModel(0)
    m.set_state(st)
    g, loss = m.grad(pairs)
    ref_loss, ref_g = torch_loss(st, pairs)
    assert abs(loss - ref_loss) <= 1e-5 * abs(ref_loss)
    groups = [(0, 512), (512, 576), (576, 4672), (4672, 4736), (4736, 4800), (4800, 4801)]
    for a, b in groups:
        scale = np.abs(ref_g[a:b]).max()
        assert np.abs(g[a:b] - ref_g[a:b]).max() <= 2e-4 * scale + 1e-9, (a, b)


def test_gradients_match_finite_differences():
    pairs = synthetic_pairs(200, 3)
    st = random_state(pairs, 4)
    m = T.WarmModel(0)
    m.set_state(st)
    g, _ = m.grad(pairs)
    rng = np.random.default_rng(5)
    idx = np.concatenate([rng.choice(512, 3, replace=False), 576 + rng.choice(4096, 4, replace=False),
                          4736 + rng.choice(64, 3, replace=False), [4800]])
    h = 1e-2
    for i in idx:
        sp, sm = st.copy(), st.copy()
        sp[i] += h
        sm[i] -= h
        m.set_state(sp)
        lp = m.grad(pairs)[1]
        m.set_state(sm)
        lm = m.grad(pairs)[1]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 2e-2 * abs(g[i]) + 2e-5, (i, fd, g[i])


def bf16(a):
    return torch.tensor(np.asarray(a, np.float32)).to(torch.bfloat16).to(torch.float32)


def test_tcgen05_gemm_inference_matches_bf16_emulation():
    """The tcgen05 GEMM that fills warm-started launches' starting depths
    (troute_warm_predict runs it on caller rows): BF16 features and weights,
    FP32 accumulation in tensor memory, the first SiLU in bf16x2 arithmetic
    (its output is the second MMA's BF16 operand), the second SiLU and the
    last layer in FP32.
    100,003 rows: a partial last 128-row tile and more tiles than resident
    CTAs. Checked against a torch emulation of that arithmetic and against the
    FP32 network."""
    pairs = synthetic_pairs(100_003, 16)
    st = random_state(pairs, 17)
    m = T.WarmModel(0)
    m.set_state(st)
    pred = m.predict(pairs[:, :8])
    assert np.isfinite(pred).all() and (pred > 0).all()
    W1, b1, W2, b2, w3, b3, mu, sd, mu_y, sd_y = unpack(st)
    x = torch.tensor(features(pairs, mu, sd))
    silu = lambda z: z / (1 + torch.exp(-z))
    t1 = bf16(bf16(x) @ bf16(W1).T + torch.tensor(b1, dtype=torch.float32)) * 0.5
    a1 = bf16(t1 + t1 * bf16(torch.tanh(t1)))    # z/2 (1 + tanh(z/2)) on bf16 values
    y = silu(a1 @ bf16(W2).T + torch.tensor(b2, dtype=torch.float32)) @ bf16(w3) + np.float32(b3)
    emu = np.exp(y.numpy().astype(np.float64) * sd_y + mu_y)
    r = np.abs(pred / emu - 1)
    print(f"\ntcgen05 GEMM inference vs emulation: median {np.median(r):.2e}, max {r.max():.2e}")
    # tanh.approx in the kernel's SiLUs against the exact one
    assert np.median(r) < 1e-2 and r.max() < 8e-2
    f1 = silu(x @ torch.tensor(W1, dtype=torch.float32).T + torch.tensor(b1, dtype=torch.float32))
    f2 = silu(f1 @ torch.tensor(W2, dtype=torch.float32).T + torch.tensor(b2, dtype=torch.float32))
    ref32 = np.exp((f2 @ torch.tensor(w3, dtype=torch.float32) + np.float32(b3)).numpy().astype(np.float64) * sd_y
                   + mu_y)
    assert np.median(np.abs(np.log(pred / ref32))) < 0.02 * sd_y


def record_pairs(net_name, seed, n_ts):
    """Pairs of a plain tight-tolerance run, on the device (torch buffer)."""
    c = synth.network(net_name, seed=seed, n_ts=n_ts)
    with T.Network(c["topo"], c["params"], cfg=tight_cfg(record_pairs=1)) as net:
        net.set_state(c["q0"], c["d0"], c["rl0"])
        st = net.run(c["qlat"])
        n = net.pairs()
        buf = torch.empty((n, 9), dtype=torch.float32, device="cuda")
        assert net.pairs(buf.data_ptr(), n) == n
    return c, st, buf


def test_pair_recording_and_training():
    c, st, buf = record_pairs("c0", None, 48)
    n_solve = st["solves"] - st["early_exits"]
    assert 0.99 * n_solve <= buf.shape[0] <= n_solve
    p = buf.cpu().numpy()
    assert (p[:, 8] > 0).all() and np.isfinite(p).all()
    m = T.WarmModel(1)
    loss = m.fit(buf.data_ptr(), buf.shape[0], epochs=12, batch=1024, lr=3e-3, seed=2)
    assert loss[-1] < 0.25 * loss[0]
    pred = m.predict(p[:, :8])
    r2 = 1 - np.var(np.log(pred) - np.log(p[:, 8])) / np.var(np.log(p[:, 8]))
    assert r2 > 0.95


@pytest.fixture(scope="module")
def c0_model():
    c, _, buf = record_pairs("c0", None, 48)
    m = T.WarmModel(11)
    m.fit(buf.data_ptr(), buf.shape[0], epochs=12, batch=1024, lr=3e-3, seed=3)
    return m


@pytest.mark.parametrize("delta,k,flags", [(0.05, 16, 0), (0.01, 4, 0), (0.05, 16, 1)])
def test_warm_routing_replays_bit_identically_in_the_oracle(c0_model, delta, k, flags):
    c = synth.network("c0", seed=77, n_ts=30)
    cfg = tight_cfg(warm_start=1, warm_k=k, record_history=1, record_start=1, schedule_flags=flags)
    with T.Network(c["topo"], c["params"], cfg=cfg) as net:
        net.set_warm_start(c0_model, delta)
        net.set_state(c["q0"], c["d0"], c["rl0"])
        st = net.run(c["qlat"])
        qh = net.history(30)
        start = net.start_history(30)
        q, d, v, rl = net.get_state()
    assert st["warm_used"] > 0.9 * (st["solves"] - st["early_exits"])
    assert np.count_nonzero(start) == st["warm_used"]
    with O.pow_mode(1):
        o = O.route_tree(c["topo"], c["params"], c["qlat"], c["q0"], c["d0"], c["rl0"], tol=TIGHT, history=True,
                         warm_start=start, warm_delta=delta, warm_k=k)
    np.testing.assert_array_equal(qh, o["q_hist"])
    np.testing.assert_array_equal(q, o["q"])
    np.testing.assert_array_equal(d, o["d"])
    np.testing.assert_array_equal(v, o["v"])
    np.testing.assert_array_equal(rl, o["reach_last"])
    assert st["iterations"] == o["iterations"]
    assert st["warm_used"] == o["warm_used"] and st["warm_fallback"] == o["warm_fallback"]


def test_warm_start_needs_a_model():
    c = synth.network("c0", n_ts=2)
    with T.Network(c["topo"], c["params"], cfg=tight_cfg(warm_start=1)) as net:
        net.set_state(c["q0"], c["d0"], c["rl0"])
        with pytest.raises(T.TrouteError):
            net.run(c["qlat"])
    with pytest.raises(T.TrouteError):
        T.Network(c["topo"], c["params"], cfg=tight_cfg(warm_start=1, mapping=2))


def _dev_stats(x, y):
    r = np.abs(x - y) / np.maximum(np.abs(y), 1e-12)
    return float(np.median(r)), float(np.quantile(r, 0.99)), float(r.max())


def test_ab_trained_network_against_plain_on_a_fresh_network():
    """Train on pairs of plain runs of one network, route a fresh-seed network
    with and without the model (two 24-step launches, rtol 1e-8):

    - the trained network must save at least 15 % of the secant passes per
      solve in the second launch, with fewer than half of its starts falling
      back. Each launch's starting depths are predicted before the launch
      from the state at its start (the launch's tcgen05 GEMM); the second
      launch starts from a routed state, the regime of the benchmark's
      launches, while the first starts from the flat initial state, where
      those features carry little (its gain is printed);
    - the plain GPU history equals the oracle's (correctly rounded powers) bit
      for bit;
    - the learned form's deviation from the plain form (median and 99th
      percentile of |dq|/q over the whole history) must not exceed twice that
      of a perfect predictor: the oracle started from the plain run's own
      converged depth of every solve, with the same bracket and pass limit.
      The reference secant stops where its bracket collapses (its two
      residuals use different X clamps, troute_mc_final.cu:86 vs :105), so any
      start other than the plain one lands elsewhere; the perfect predictor
      already deviates by more than 1e-6 at the 99th percentile, which is why
      "discharge within 1e-6 of the plain form" is out of reach for any warm
      start, learned or not. The plain form's own one-ulp sensitivity (initial
      depth moved by one ulp; C-library vs correctly rounded pow) is printed
      beside it."""
    _, _, buf = record_pairs("tree:100000", 31, 24)
    m = T.WarmModel(5)
    loss = m.fit(buf.data_ptr(), buf.shape[0], epochs=4, batch=8192, lr=2e-3, seed=6)
    assert loss[-1] < loss[0]
    c = synth.network("tree:100000", seed=32, n_ts=48)
    out = {}
    for warm in (0, 1):
        cfg = tight_cfg(warm_start=warm, record_history=1)
        with T.Network(c["topo"], c["params"], cfg=cfg) as net:
            if warm:
                net.set_warm_start(m, 0.05)
            net.set_state(c["q0"], c["d0"], c["rl0"])
            st1 = net.run(c["qlat"][:24])
            h1 = net.history(24)
            st2 = net.run(c["qlat"][24:])
            out[warm] = (st1, st2, np.concatenate([h1, net.history(24)]))
    per_solve = lambda st: st["iterations"] / (st["solves"] - st["early_exits"])
    ip1, iw1 = per_solve(out[0][0]), per_solve(out[1][0])
    plain, warm = out[0][1], out[1][1]
    n_solve = plain["solves"] - plain["early_exits"]
    ip, iw = per_solve(plain), per_solve(warm)
    fb = warm["warm_fallback"] / max(1, warm["warm_used"])
    qw, qp = out[1][2], out[0][2]
    learned = _dev_stats(qw, qp)

    def oracle_hist(mode=1, d0=None, **kw):
        with O.pow_mode(mode):
            return O.route_tree(c["topo"], c["params"], c["qlat"], c["q0"], c["d0"] if d0 is None else d0, c["rl0"],
                                tol=TIGHT, history=True, threads=16, **kw)

    with O.pow_mode(1):
        o = O.route_tree(c["topo"], c["params"], c["qlat"], c["q0"], c["d0"], c["rl0"], tol=TIGHT, history=True,
                         depth_history=True, threads=16)   # all 48 steps
    np.testing.assert_array_equal(qp, o["q_hist"])
    perfect = _dev_stats(oracle_hist(warm_start=o["d_hist"], warm_delta=0.05, warm_k=16)["q_hist"], o["q_hist"])
    ulp = _dev_stats(oracle_hist(d0=np.nextafter(c["d0"], np.inf))["q_hist"], o["q_hist"])
    libm = _dev_stats(oracle_hist(mode=0)["q_hist"], o["q_hist"])
    print(f"\nA/B tree:100000 seed 32, second 24-step launch: plain {ip:.3f} it/solve, warm {iw:.3f} it/solve "
          f"({100 * (1 - iw / ip):.1f} % fewer), fallback {fb:.3f}; first launch (from the flat initial state): "
          f"plain {ip1:.3f}, warm {iw1:.3f} ({100 * (1 - iw1 / ip1):.1f} % fewer)\n"
          f"  |dq|/q vs plain (median, p99, max): learned {learned[0]:.2e} {learned[1]:.2e} {learned[2]:.2e}; "
          f"perfect predictor {perfect[0]:.2e} {perfect[1]:.2e} {perfect[2]:.2e}; "
          f"plain with initial depth +1 ulp {ulp[0]:.2e} {ulp[1]:.2e} {ulp[2]:.2e}; "
          f"plain with C-library pow {libm[0]:.2e} {libm[1]:.2e} {libm[2]:.2e}")
    assert warm["warm_used"] > 0.9 * n_solve
    assert fb < 0.5
    assert iw <= 0.85 * ip
    assert learned[0] <= 2.0 * perfect[0] and learned[1] <= 2.0 * perfect[1]
    assert perfect[1] > 1e-6
