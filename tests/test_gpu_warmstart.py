"""The learned warm start: device tensor generator, the MLP's forward pass and gradients
against the CPU oracle, training, and the gain of the trained network over random init.

Gradient tolerance: the device accumulates in FP32 and rounds activations to BF16 where the
oracle (FP64 accumulation of the same BF16 operands) may round a value near a BF16 tie the
other way; per parameter block the relative Frobenius difference stays below 2e-2 and the
cosine similarity above 0.999.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def built(pkg):
    import __graft_entry__

    __graft_entry__.build()
    return pkg


@pytest.fixture(scope="module")
def mlp_oracle():
    import mlp_oracle

    return mlp_oracle


def test_synth_matches_host_reconstruction(built, oracle):
    import torch

    dims, R = (13, 11, 7), 4
    rng = np.random.default_rng(0)
    buf = torch.zeros(int(np.prod(dims)), dtype=torch.float32, device="cuda")
    facs, w = built.warmstart.synth_device(dims, R, 0.3, -2000.0, rng, buf.data_ptr())
    T = np.reshape(buf.cpu().numpy(), dims, order="F")
    ref = oracle.reconstruct(facs, w)
    assert np.linalg.norm(T - ref) / np.linalg.norm(ref) < 1e-6
    # noise at 20 dB: ||noise|| / ||signal|| = 0.1 within sampling error
    big = (64, 64, 64)
    buf2 = torch.zeros(int(np.prod(big)), dtype=torch.float32, device="cuda")
    rng = np.random.default_rng(1)
    facs, w = built.warmstart.synth_device(big, R, 0.3, 20.0, np.random.default_rng(1), buf2.data_ptr(), seed=7)
    noisy = buf2.cpu().numpy().astype(np.float64)
    clean = oracle.reconstruct(facs, w).reshape(-1, order="F")
    noise = noisy - clean
    assert abs(np.linalg.norm(noise) / np.linalg.norm(clean) - 0.1) < 2e-3
    assert abs(noise.mean()) < 4.0 * noise.std() / np.sqrt(noise.size)
    # deterministic for a seed
    buf3 = torch.zeros_like(buf2)
    built.warmstart.synth_device(big, R, 0.3, 20.0, np.random.default_rng(1), buf3.data_ptr(), seed=7)
    assert torch.equal(buf2, buf3)


WIDTHS = (96, 64, 80, 48)


def test_mlp_forward_and_gradients_match_oracle(built, mlp_oracle):
    rng = np.random.default_rng(2)
    p = mlp_oracle.init_params(WIDTHS, rng)
    p[WIDTHS[1] * WIDTHS[0]:WIDTHS[1] * WIDTHS[0] + WIDTHS[1]] = rng.uniform(-0.1, 0.1, WIDTHS[1])  # nonzero b1
    x = rng.standard_normal((24, WIDTHS[0])).astype(np.float32)
    t = rng.standard_normal((24, WIDTHS[3])).astype(np.float32)
    net = built.WarmStartMLP(WIDTHS, params=p)
    y = net.forward(x)
    y_ref, _ = mlp_oracle.forward(p, WIDTHS, x)
    assert np.linalg.norm(y - y_ref) / np.linalg.norm(y_ref) < 1e-2
    loss, g = net.gradients(x, t)
    loss_ref, g_ref = mlp_oracle.loss_and_gradients(p, WIDTHS, x, t)
    assert abs(loss - loss_ref) / loss_ref < 1e-2
    blocks = mlp_oracle.split_params(np.arange(g.size), WIDTHS)
    for name, ix in zip(["W1", "b1", "W2", "b2", "W3", "b3"], blocks):
        ix = np.asarray(ix).ravel()
        a, b = g[ix].astype(np.float64), g_ref[ix]
        rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        cos = float(a @ b / (np.linalg.norm(a) * np.linalg.norm(b) + 1e-300))
        assert rel < 2e-2 and cos > 0.999, (name, rel, cos)
    net.close()


def test_mlp_training_reduces_loss(built):
    rng = np.random.default_rng(3)
    A = rng.standard_normal((WIDTHS[0], WIDTHS[3])) / np.sqrt(WIDTHS[0])
    X = rng.standard_normal((2048, WIDTHS[0])).astype(np.float32)
    T = np.tanh(X @ A).astype(np.float32)
    net = built.WarmStartMLP(WIDTHS, seed=4)
    losses = net.fit(X, T, epochs=20, batch=128, lr=2e-3)
    assert losses[-20:].mean() < 0.25 * losses[:5].mean()
    net.close()


def _prepare(built, eng, core_eng, dims, R, omegas, seed, buf):
    rng = np.random.default_rng(seed)
    facs, w = built.warmstart.synth_device(dims, R, float(rng.uniform(0, 0.8)), float(rng.uniform(15, 40)), rng,
                                           buf.data_ptr())
    eng.set_tensor_device(buf.data_ptr(), keepalive=buf)
    core_eng.set_tensor_device(buf.data_ptr(), keepalive=buf)
    nrm = float(buf.double().norm())
    Qs, _ = built.warmstart.sketch_bases(built.warmstart.sketch(eng, omegas))
    G = built.warmstart.core(core_eng, Qs)
    prop = built.warmstart.jennrich(G, R, np.random.default_rng(seed + 7))
    return nrm, Qs, G, prop


def test_core_als_follows_the_oracle(built, oracle):
    # the teacher: batched ALS on S^3 cores from the Jennrich proposals, against the oracle's
    # FP64 ALS on the same core from the same start (fixed sweeps, unit columns, signs of the start)
    rng = np.random.default_rng(11)
    S, R = 8, 5
    cores, props = [], []
    for t in range(6):
        G, _, _ = oracle.lowrank_plus_noise((S, S, S), R, 0.3, 30.0, rng)
        cores.append(G.astype(np.float64))
        props.append(built.warmstart.jennrich(G.astype(np.float64), R, np.random.default_rng(t)))
    with built.BatchEngine([(S, S, S)] * len(cores), [R] * len(cores), [1.0] * len(cores)) as be:
        got, sweeps = built.warmstart.core_als(be, cores, props, 4)
    assert np.all(sweeps == 4)
    for G, P, C in zip(cores, props, got):
        Gf = np.asarray(G, dtype=np.float32).astype(np.float64)
        chk = oracle.FitCheck(0.0, 4, float(np.linalg.norm(Gf)))
        F, lam, _, _ = oracle.als_optimize(Gf, [p.copy() for p in P], np.ones(R), check=chk)
        for Fn, Cn, Pn in zip(F, C, P):
            assert np.allclose(np.linalg.norm(Cn, axis=0), 1.0)
            assert np.all(np.sum(Cn * Pn, axis=0) >= 0)  # signed like the start
            sg = np.sign(np.sum(Fn * Pn, axis=0))
            sg[sg == 0] = 1.0
            # FP32 products in the batched MTTKRP: agreement to ~1e-6 per sweep, amplified by
            # the conditioning of the normal equations over four sweeps
            assert np.max(np.abs(Fn * sg - Cn)) < 1e-3


def test_warm_start_gain_over_random_init(built):
    # A small instance of the warm-start workload: 32^3 FP32, rank 6, a sketch of 6 columns
    # per mode.  The batched solver runs ALS on the 200 training cores from their proposals
    # (one sweep: the network's input step; to convergence: its target); the network is
    # judged on 16 held-out tensors by the sweeps ALS needs to reach 99% of the best fit any
    # start attains: against random init (the reference's start), the proposal, and the
    # proposal after one core sweep (the network's input alone).  Asserted: the learned start
    # beats random init on the median, the starts lie in the sketched column range with unit
    # columns, and ALS from the learned start ends as well as from random init (ALS still
    # decides the result).
    import torch

    ws = built.warmstart
    dims, R, S = (32, 32, 32), 6, 6
    omegas = ws.gaussian_test_matrices(dims, S, seed=99)
    buf = torch.zeros(int(np.prod(dims)), dtype=torch.float32, device="cuda")
    with built.Engine(dims, R, dtype=np.float32, precision="bf16x3") as eng, \
            built.Engine(dims, S * S, dtype=np.float32, precision="bf16x3") as core_eng:
        Gs, props = [], []
        for s in range(200):
            _, _, G, prop = _prepare(built, eng, core_eng, dims, R, omegas, s, buf)
            Gs.append(G)
            props.append(prop)
        with built.BatchEngine([(S, S, S)] * len(Gs), [R] * len(Gs), [1.0] * len(Gs)) as be:
            P1, _ = ws.core_als(be, Gs, props, 1)
            Ps, _ = ws.core_als(be, Gs, props, 300, tol=1e-8)
        steps = [[a - b for a, b in zip(p1, p)] for p1, p in zip(P1, props)]
        scale = float(np.sqrt(np.mean([np.mean(np.square(d)) for D in steps for d in D])))
        X, Y = ws.features(props, steps, scale), ws.targets(props, Ps, scale)
        net = built.WarmStartMLP((6 * S * R, 256, 256, S * R), seed=5)
        net.step_scale = scale
        net.step_gain = ws.fit_step_gain(X[:-60], Y[:-60], S * R)
        Yr = ws.residual_targets(X, Y, S * R, net.step_gain)
        losses = net.fit(X[:-60], Yr[:-60], epochs=60, batch=64, lr=1e-3)
        assert losses[-10:].mean() < losses[:3].mean()
        assert 0.0 <= net.calibrate(X[-60:], Yr[-60:]) <= 1.0
        sw = {"random": [], "proposal": [], "one_core_sweep": [], "warm": []}
        final = {"random": [], "warm": []}
        with built.BatchEngine([(S, S, S)], [R], [1.0]) as be1:
            for s in range(5000, 5016):
                nrm, Qs, G, prop = _prepare(built, eng, core_eng, dims, R, omegas, s, buf)
                (p1,), _ = ws.core_als(be1, [G], [prop], 1)
                Fw = ws.warm_factors(net, Qs, prop, [a - b for a, b in zip(p1, prop)])
                Fp = ws.lift(Qs, prop)
                F1 = ws.lift(Qs, p1)
                for F in (Fw, Fp, F1):
                    if F is None:
                        continue
                    for Fn, Q in zip(F, Qs):  # inside the sketched column range, unit columns
                        assert np.linalg.norm(Fn - Q @ (Q.T @ Fn)) < 1e-8 * np.sqrt(Fn.size)
                        assert np.allclose(np.linalg.norm(Fn, axis=0), 1.0)
                fallback = built.random_factors(dims, R, np.random.default_rng(1))[0]
                starts = {"random": built.random_factors(dims, R, np.random.default_rng(20_000 + s))[0],
                          "proposal": Fp if Fp is not None else fallback,
                          "one_core_sweep": F1 if F1 is not None else fallback,
                          "warm": Fw if Fw is not None else fallback}
                trajs = {}
                for key, F0 in starts.items():
                    eng.set_factors(F0, np.ones(R))
                    trajs[key] = eng.optimize(built.api._to_device_check(built.FitCheck(0.0, 60, nrm)))
                target = 0.99 * max(t.max() for t in trajs.values())
                for key in sw:
                    sw[key].append(ws.sweeps_to_fit(trajs[key], target) or 61)
                final["random"].append(trajs["random"][-1])
                final["warm"].append(trajs["warm"][-1])
        med = {k: float(np.median(v)) for k, v in sw.items()}
        mean = {k: float(np.mean(v)) for k, v in sw.items()}
        print("sweeps to 99% of the best fit: median", med, "mean", mean, "| final fit (median): random",
              np.median(final["random"]), "learned", np.median(final["warm"]))
        assert med["warm"] < med["random"]
        assert np.median(final["warm"]) >= np.median(final["random"]) - 1e-2
        net.close()
