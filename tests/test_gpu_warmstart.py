"""The learned warm start on the GPU, through the C ABI:

* the network's forward pass, loss and parameter gradients (hand-written CUDA
  kernels) against torch's CPU conv3d autograd in float64;
* the resampling kernels (features, targets) and the warm-start
  initialisation against the numpy restatement in oracle/warmstart_ref.py;
* training lowers the loss; the windowed convergence run and its fallback
  to the reference's schedule (which must then give exactly the plain run's
  KPIs).
"""
import numpy as np
import pytest

from airboxcalc_gb300 import airboxgen as ag
from airboxcalc_gb300 import engine as E
from airboxcalc_gb300 import warmstart as W
from oracle import warmstart_ref as R_

pytestmark = pytest.mark.gpu

SMALL = dict(Lx=130.37, Ly=95.29, Lz=110.53, t=3.11, d_in=40.3, stub=21.7, pleat=40.0, dx=5.0,
             baffle={"z": 50.19, "x0": 3.11, "x1": 60.07, "y0": 70.21})
RUN = dict(K=3, aniso=10, u=0.06, tau=0.51, steps=60, avg=20, every=30)


def geometry(spec=None):
    spec = spec or ag.AirboxSpec(**SMALL)
    return E.prepare({"tris": ag.build_airbox(spec), **spec.prepare_params()})


def _torch():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    return torch


# float32 convolutions: against the float64 network, to float32 rounding.
#
# Tensor cores (bf16 operands, float32 accumulation): each convolution is exact to float32 summation error when its
# operands are bf16 values (tests/native/conv_tc_check.cu, through test_gpu_conv_tc.py).  Through the whole network
# no tight bound exists: a float32 sum that lands within its rounding error of a bf16 rounding boundary rounds the
# other way than the float64 sum does (one bf16 unit, 0.4 %), the change spreads to the next layers' sums and tips
# more of them, and pre-activations near zero then cross the ReLU, which switches whole gradient entries on or off.
# Depending on the data this stays at float32 level or reaches a few per mille in the prediction and a few
# per cent in a layer's parameter gradient (measured on six seeds at 8^3 to 16^3).  So the prediction and loss
# are checked against the exact network to bf16 rounding, and the gradients against the network whose
# convolutions round the same operands to bf16 (which removes the systematic part): every tensor within 15 %
# relative L2 and the whole gradient within 5 %; a missing term of the backward pass (a skip connection, a mask,
# an accumulation) is an error of order one.
TOL = {False: dict(pred=1e-4, loss=1e-5, grad=1e-4), True: dict(pred=3e-2, loss=3e-2, grad=0.15, grad_all=0.05)}

@pytest.mark.parametrize("tc", [False, True])
@pytest.mark.parametrize("res,base,levels,coords", [(8, 8, 2, False), (16, 8, 3, False), (8, 8, 2, True),
                                                    (32, 8, 2, False)])
def test_network_gradients_match_torch_autograd(res, base, levels, coords, tc):
    torch = _torch()
    net = W.Net(res, base, levels, seed=3, coords=coords)
    net.set_tensor_cores(tc)
    assert net.info["tensor_cores"] == int(tc)
    tol = TOL[tc]
    w = net.get_weights()
    assert w.size == net.n_params and net.info["in_channels"] == net.n_in
    rng = np.random.default_rng(1)
    B = 2
    x = rng.standard_normal((B, net.n_in, res, res, res)).astype(np.float32)
    t = rng.standard_normal((B, 4, res, res, res)).astype(np.float32)
    m = rng.uniform(0, 1, (B, res, res, res)).astype(np.float32)
    scale = 1.0 / (4 * float(m.sum()))
    dx, dt, dm = (torch.from_numpy(a).cuda() for a in (x, t, m))
    dpred = torch.empty((B, 4, res, res, res), dtype=torch.float32, device="cuda")
    dgrad = torch.empty(net.n_params, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    loss = net.forward_backward(dx.data_ptr(), dt.data_ptr(), dm.data_ptr(), B, scale, dpred.data_ptr(),
                                dgrad.data_ptr())
    pred, grad = dpred.cpu().numpy(), dgrad.cpu().numpy()

    X, T, M = (torch.tensor(a, dtype=torch.float64) for a in (x, t, m))
    with torch.no_grad():
        P = R_.net_forward(R_.unpack(w, base, levels, torch, net.n_in), X, levels, torch)
        L = scale * (M[:, None] * (P - T) ** 2).sum()
    assert np.abs(pred - P.numpy()).max() <= tol["pred"] * np.abs(P.numpy()).max()
    assert abs(loss - L.item()) <= tol["loss"] * abs(L.item())
    layers = R_.unpack(w, base, levels, torch, net.n_in)
    P = R_.net_forward(layers, X, levels, torch, bf16_operands=tc)
    L = scale * (M[:, None] * (P - T) ** 2).sum()
    L.backward()
    off, refs = 0, []
    for i, (wt, bs, s, relu) in enumerate(layers):
        for ref in (wt.grad.numpy().ravel(), bs.grad.numpy().ravel()):
            got = grad[off:off + ref.size]
            off += ref.size
            refs.append(ref)
            err = np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-30)
            assert err < tol["grad"], f"layer {i}: relative gradient error {err:.2e}"
    assert off == grad.size
    ref = np.concatenate(refs)
    assert np.linalg.norm(grad - ref) / np.linalg.norm(ref) < tol.get("grad_all", tol["grad"])


@pytest.mark.parametrize("coords", [False, True])
def test_features_and_targets_match_restatement(coords):
    g = geometry()
    net = W.Net(16, 8, 2, coords=coords)
    S = E.Simulation(g, RUN)
    S.run()
    net.add_sample(S)
    x, t, m = net.sample(0)
    fx, _ = net.predict(S)
    assert np.array_equal(x, fx)
    cls = R_.classes(g)
    rx, dist = R_.features(cls, 16, RUN["K"], coords)
    assert x.shape[0] == rx.shape[0] == (12 if coords else 9)
    for c in (0, 1, 2, 3, 5, 6, 7, 8) + ((9, 10, 11) if coords else ()):
        assert np.array_equal(x[c], rx[c]), f"feature channel {c}"
    assert (cls == 2).any() and (cls == 4).any()
    # jump flooding against the exact distance transform
    d = np.abs(x[4] - rx[4])
    assert (d < 1e-6).mean() > 0.97 and d.max() < 0.1
    # targets: footprint means of the time-averaged fields
    acc = S.get_acc().reshape(4, -1)
    fl = g.fluid.reshape(g.nx, g.ny, g.nz).astype(bool)
    avg = {}
    for c, k in enumerate(("ux", "uy", "uz", "rho")):
        a = np.zeros((g.nx, g.ny, g.nz))
        a[fl] = acc[c]
        avg[k] = a
    rt, rm = R_.targets(cls, avg, 16, RUN["u"])
    assert np.allclose(m, rm, rtol=0, atol=1e-6)
    assert np.abs(t - rt).max() < 2e-4 * max(1.0, np.abs(rt).max())


@pytest.mark.parametrize("storage,tol", [("f32", 2e-6), ("f32exact", 2e-6), ("f16", 2e-4), ("bf16", 2e-3)])
def test_warm_start_populations_match_restatement(storage, tol):
    g = geometry()
    net = W.Net(16, 8, 2, seed=7)
    # make the prediction non-trivial: scale the head so |u| reaches a few u0
    w = net.get_weights()
    w[-(4 * 8 * 27 + 4):] *= 20.0
    net.set_weights(w)
    S = E.Simulation(g, dict(RUN, storage=storage, allowBf16=True))
    feats, pred = net.predict(S)
    W.warm_start(S, net)
    f = S.get_f().reshape(19, -1)
    ijk = np.argwhere(g.fluid.reshape(g.nx, g.ny, g.nz))
    ref = R_.apply(pred.astype(np.float64), feats[0].astype(np.float64), ijk, (g.nx, g.ny, g.nz), RUN["u"])
    assert np.abs(f - ref).max() < tol
    assert np.abs(ref[0] - 1 / 3).max() > 1e-4          # the start differs from f = w_i
    assert S.refresh().step == 0 and S.info.nacc == 0


def test_training_lowers_the_loss():
    _torch()
    net = W.Net(16, 8, 2, seed=11)
    for s in (3, 4, 5):
        spec = ag.random_spec(s, dx=4.0)
        g = geometry(spec)
        S = E.Simulation(g, dict(RUN, steps=200, avg=100, every=100))
        S.run()
        net.add_sample(S)
    assert net.info["n_samples"] == 3
    before = net.eval_loss(0, 3)
    hist = net.train(0, 3, 60, batch=2, lr=3e-3, lr_min=1e-4, seed=1, flip=True)
    after = net.eval_loss(0, 3)
    assert np.all(np.isfinite(hist))
    assert after < 0.3 * before, (before, after, hist[-5:])


def test_converge_and_fallback_to_the_reference_schedule():
    g = geometry()
    net = W.Net(16, 8, 2, seed=5)
    S = E.Simulation(g, RUN)
    W.warm_start(S, net)
    r = W.converge(S, settle=20, window=20, min_avg=40, max_steps=400, tol=0.5)
    assert r["converged"] and r["steps"] % 20 == 0 and r["windows"] >= 2 and r["steps"] >= 60
    assert all(np.isfinite(v) for v in r["metrics"].values())
    # a stop rule that cannot fire: the run falls back to f = w_i and the full schedule
    S2 = E.Simulation(g, RUN)
    res = W.solve_warm(S2, net, settle=10, window=20, min_avg=20, max_steps=50, tol=1e-14)
    assert res["fell_back"] and res["warm_steps"] == 50 and res["steps"] == RUN["steps"]
    plain = E.simulate(g, RUN)["metrics"]
    for k in ("gamma", "gammaCore", "zeta", "maxToMean"):
        assert res["metrics"][k] == plain[k], k
    assert res["total_ms"] >= res["infer_ms"] > 0


def test_standard_error_stop_rule():
    """ABX_RULE_STDERR: the windows' own KPIs (evaluated from the running sums minus a snapshot taken at the
    window's start) give the batch-means standard error the rule compares with tol / 2.  A twin simulation that
    restarts its averages at every window reproduces the windows' KPIs, and from them the same standard error."""
    g = geometry()
    net = W.Net(16, 8, 2, seed=5)
    rule = dict(settle=20, window=20, min_avg=40, max_steps=140, tol=1e-12, rule=1, min_windows=3)
    S = E.Simulation(g, RUN)
    W.warm_start(S, net)
    r = W.converge(S, **rule)
    assert not r["converged"] and r["steps"] == 140 and r["windows"] == 6
    T = E.Simulation(g, RUN)
    W.warm_start(T, net)
    T.step(20)
    wg, wz = [], []
    for _ in range(6):
        T.clear_acc()
        T.step(20, True)
        m = T.evaluate()["metrics"]
        wg.append(m["gammaCore"])
        wz.append(m["zeta"])
    run_g, run_z = r["metrics"]["gammaCore"], r["metrics"]["zeta"]
    se = max(np.std(wg, ddof=1) / np.sqrt(6) / abs(run_g), np.std(wz, ddof=1) / np.sqrt(6) / abs(run_z))
    assert r["change"] == pytest.approx(se, rel=1e-3)
    # a loose tolerance fires once min_windows windows and min_avg steps are in
    S2 = E.Simulation(g, RUN)
    W.warm_start(S2, net)
    r2 = W.converge(S2, **dict(rule, tol=10.0))
    assert r2["converged"] and r2["windows"] == 3 and r2["change"] <= 5.0


def test_net_argument_errors():
    with pytest.raises(E.AirboxError):
        W.Net(12, 8, 2)            # not a power of two
    with pytest.raises(E.AirboxError):
        W.Net(16, 12, 2)           # base not a multiple of 8
    with pytest.raises(E.AirboxError):
        W.Net(8, 8, 4)             # 8 / 2^3 < 2
    net = W.Net(8, 8, 2)
    g = geometry()
    S = E.Simulation(g, RUN)
    with pytest.raises(E.AirboxError):
        net.add_sample(S)          # no averages yet
    with pytest.raises(E.AirboxError):
        net.train(0, 1, 1)         # no samples


# D3Q19 velocities in the library's population order (src/engine.js:4-12).
CX = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0])
CY = np.array([0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1])
CZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1])


def test_trained_network_beats_the_uniform_start():
    """What the shipped, trained network gains over the same method without it, on held-out airboxes
    (seeds 6000-6011 of the generator at dx 2 mm; training used seeds 0-3999):

    * its start is much closer to the plain float32 run's time-averaged velocity than the uniform start
      f = w_i, whose velocity is zero (relative L2 error exactly 1);
    * the same float16 convergence run (default stop rule) ends with smaller gamma core / zeta errors
      against the plain float32 run on the reference's 6000/2000 schedule when it starts from the network's
      prediction (abx_sim_solve_warm) than when it starts from f = w_i (abx_sim_converge after a reset).

    Measured with the shipped network (11 stable airboxes): start error 0.19-0.29 (median 0.25); KPI error after
    the run median 1.5 % warm against 12 % uniform; 4 warm runs and no uniform run within 1 %.  The bounds leave
    room for rounding differences between GPUs, not for a network that stopped helping.
    """
    net = W.Net.load()
    start_err, warm_err, uniform_err = [], [], []
    for seed in range(6000, 6012):
        spec, K = W.variant(seed)
        run = dict(W.RUN, K=K)
        try:
            g = E.prepare({"tris": ag.build_airbox(spec), **spec.prepare_params(), "maxCells": 1e10})
            P = E.Simulation(g, run)
            P.run()
        except E.AirboxError:        # leaking or unstable draws have no reference result
            continue
        ref = P.evaluate()["metrics"]
        ubar = P.get_acc().reshape(4, P.NF)[:3].astype(np.float64)
        del P
        S = E.Simulation(g, dict(run, storage="f16"))
        W.warm_start(S, net)
        f = S.get_f().reshape(19, S.NF).astype(np.float64)
        u0 = np.stack([CX @ f, CY @ f, CZ @ f]) / f.sum(0)
        start_err.append(np.linalg.norm(u0 - ubar) / np.linalg.norm(ubar))

        def err(m):
            return max(abs(m[k] - ref[k]) / abs(ref[k]) for k in ("gammaCore", "zeta"))

        warm_err.append(err(W.solve_warm(S, net)["metrics"]))
        S.reset()
        uniform_err.append(err(W.converge(S)["metrics"]))
        del S, g
    print("start error", np.round(start_err, 3), "\nwarm KPI error", np.round(warm_err, 4),
          "\nuniform KPI error", np.round(uniform_err, 4))
    assert len(warm_err) >= 6, "too few stable held-out airboxes"
    assert np.median(start_err) < 0.35, start_err
    assert np.median(warm_err) < 0.25 * np.median(uniform_err), (warm_err, uniform_err)
    n_warm, n_uniform = sum(e < 0.01 for e in warm_err), sum(e < 0.01 for e in uniform_err)
    assert n_warm >= 3 and n_warm > n_uniform, (warm_err, uniform_err)
