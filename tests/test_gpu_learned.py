"""The learned acceptance criterion: the GPU's own forward/backward kernels
against the FP64 CPU restatement, the traversal's fused (mma.sync) inference
against the same, and the end-to-end pipeline -- pairs labelled by the plain
walk at theta = 0.5, training on the GPU, and what the trained network gains
over the theta criterion without it, measured against the FP64 direct sum."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import DT, G, ROOT, THETA, assert_bits_equal

pytestmark = pytest.mark.gpu
SIMULATE = ROOT / "barnes-hut_gb300" / "_build" / "simulate"


def he_params(rng):
    from oracle import mlp
    p = np.zeros(mlp.NPARAMS, np.float32)
    p[mlp.OFF_W1:mlp.OFF_B1] = rng.normal(0, np.sqrt(2 / 8), 512)
    p[mlp.OFF_B1:mlp.OFF_W2] = rng.normal(0, 0.1, 64)
    p[mlp.OFF_W2:mlp.OFF_B2] = rng.normal(0, np.sqrt(2 / 64), 4096)
    p[mlp.OFF_B2:mlp.OFF_W3] = rng.normal(0, 0.1, 64)
    p[mlp.OFF_W3:mlp.OFF_B3] = rng.normal(0, np.sqrt(1 / 64), 64)
    p[mlp.OFF_B3] = 0.3
    return p


def test_gradient_matches_cpu_fp64(bh):
    from oracle import mlp
    rng = np.random.default_rng(0)
    p = he_params(rng)
    X = rng.normal(0, 1, (2000, 8)).astype(np.float32)
    T = rng.normal(0, 1, 2000).astype(np.float32)
    loss_gpu, g_gpu = bh.mlp_gradient(p, X, T)
    loss_cpu, g_cpu = mlp.loss_and_grad(p, X, T)
    # Tolerance: FP32 accumulation on the GPU against FP64 on the CPU, with
    # the same BF16 roundings: 1e-4 relative on the loss, 2e-3 on the
    # gradient vector, 1e-2 per block of parameters.
    assert abs(loss_gpu - loss_cpu) <= 1e-4 * loss_cpu
    assert np.linalg.norm(g_gpu - g_cpu) <= 2e-3 * np.linalg.norm(g_cpu)
    for lo, hi in ((mlp.OFF_W1, mlp.OFF_B1), (mlp.OFF_B1, mlp.OFF_W2), (mlp.OFF_W2, mlp.OFF_B2),
                   (mlp.OFF_B2, mlp.OFF_W3), (mlp.OFF_W3, mlp.OFF_B3)):
        assert np.linalg.norm(g_gpu[lo:hi] - g_cpu[lo:hi]) <= 1e-2 * np.linalg.norm(g_cpu[lo:hi]) + 1e-12
    assert abs(g_gpu[mlp.OFF_B3] - g_cpu[mlp.OFF_B3]) <= 1e-3 * abs(g_cpu[mlp.OFF_B3]) + 1e-7


def test_fused_inference_matches_cpu(bh):
    from oracle import mlp
    rng = np.random.default_rng(1)
    p = he_params(rng)
    mean = rng.normal(0, 1, 8).astype(np.float32)
    inv_std = rng.uniform(0.5, 2.0, 8).astype(np.float32)
    scale = np.concatenate([mean, inv_std, np.full(8, -3.0, np.float32), np.full(8, 3.0, np.float32),
                            np.array([-6.0, 2.0], np.float32)])
    F = (mean + rng.normal(0, 1, (1000, 8)) / inv_std).astype(np.float32)
    y, inr = bh.mlp_predict(p, scale, F)
    Z = np.clip((F - mean) * inv_std, -64, 64).astype(np.float32)
    ycpu, _ = mlp.forward(p, Z)
    ycpu = ycpu * 2.0 - 6.0
    d = np.abs(y - ycpu)
    # BF16 rounding of hidden activations computed in different FP32 orders
    # can move a value by one BF16 ulp; the outputs agree to 2e-2 worst case.
    assert np.median(d) < 1e-4 and d.max() < 2e-2
    z = (F - mean) * inv_std
    assert np.array_equal(inr, np.all((z >= -3) & (z <= 3), axis=1))


def _system(bh, seed, n):
    pos, vel, mass, ids = bh.generate_system(seed, n, 0.1, 0.05)
    c = bh.Context(n)
    c.set_bodies(pos, vel, mass, ids)
    c.compute_bbox(); c.compute_keys(); c.sort_bodies(); c.build_tree()
    return c


def test_learned_pipeline_what_the_network_gains(bh):
    """Pairs labelled by the plain walk at theta = 0.5 on three 60k systems,
    the network trained on the GPU, then on an unseen system:

    * the network predicts the candidates' errors more tightly than the
      analytic estimate G m s^2 / d_min^4 it refines (the 5-95 % band of the
      residuals);
    * at the same per-body budget, the criterion that asks the network about
      the candidates near the allowance is as accurate as the analytic
      estimate alone (median within 5 %) with at most 5 % more interactions
      (on this 60k system the network decides few candidates; on the 4M
      system the bench compares the two at every budget);
    * against the method without it it makes fewer interactions than the
      theta test at 1.05, and than every wider theta of a sweep (1.3-2.5)
      whose median error is at most its own; the bodies' errors stay within
      their budget.

    What it does not gain, measured in the bench and stated in the design:
    a plain theta test at a wider angle is faster at equal error on this
    walk (the walk's per-node cost, not the interactions, bounds it there)."""
    feats, labels = [], []
    for seed in (101, 102, 103):
        with _system(bh, seed, 60_000) as c:
            f, lab = c.learned_collect(THETA, 0.5, 3.0, G, max_pairs=1_500_000)
            ok = np.all(np.isfinite(f), axis=1) & np.isfinite(lab)
            feats.append(f[ok]); labels.append(lab[ok])
    F = np.concatenate(feats); L = np.concatenate(labels)
    assert len(L) > 50_000
    params, scale, losses = bh.mlp_train(F, L, epochs=8, batch=2048, lr=2e-3, seed=0)
    # standardised MSE (1.0 = predicting the mean): the network learns the labels
    assert losses[-1] < 0.3 and losses[-1] < losses[0]
    with _system(bh, 104, 60_000) as c:
        f, lab = c.learned_collect(THETA, 0.5, 3.0, G, max_pairs=400_000)
        ok = np.all(np.isfinite(f), axis=1) & np.isfinite(lab)
        f, lab = f[ok], lab[ok]
        pred, inr = bh.mlp_predict(params, scale, f)
        r_net = (lab - pred)[inr]
        r_ana = lab - (f[:, 3] + 2.0 * f[:, 1])
        band = lambda r: float(np.percentile(r, 95) - np.percentile(r, 5))  # noqa: E731
        print(f"residual 5-95 % band: network {band(r_net):.3f}, analytic {band(r_ana):.3f} decades")
        assert inr.mean() > 0.95
        assert band(r_net) < 0.9 * band(r_ana)

        rng = np.random.default_rng(2)
        sample = np.sort(rng.choice(c.n, 1024, replace=False))
        ref = c.direct_sum(sample, G)
        rel = lambda a: np.linalg.norm(a[sample] - ref, axis=1) / np.linalg.norm(ref, axis=1)  # noqa: E731
        e_theta = rel(c.compute_accelerations(THETA, G, 0.0, bh.MODE_FP32_FAR))
        n_theta = c.interaction_count()
        # the method without the network over a theta sweep (the reference's
        # test, traversal.cpp:78, at wider angles)
        sweep = []
        for th in (1.05, 1.3, 1.6, 2.0, 2.5):
            e = rel(c.compute_accelerations(th, G, 0.0, bh.MODE_FP32_FAR))
            sweep.append((float(np.median(e)), c.interaction_count(), th))
        rows = {}
        for budget in (1e-6, 1e-5):
            for name, b in (("network", 0.5), ("analytic", 0.0)):
                c.learned_set_model(params, scale, budget=budget, theta_max=3.0)
                c.learned_set_criterion(b, 0.25)
                e = rel(c.compute_accelerations(THETA, G, 0.0, bh.MODE_LEARNED))
                rows[(budget, name)] = (float(np.median(e)), c.interaction_count(), c.learned_stats(), e)
    print(f"theta {THETA}: median {np.median(e_theta):.3g}, {n_theta} interactions")
    for budget in (1e-6, 1e-5):
        med_n, n_n, st, e_n = rows[(budget, "network")]
        med_a, n_a, _, _ = rows[(budget, "analytic")]
        print(f"budget {budget:g}: network median {med_n:.3g} / {n_n} interactions, analytic {med_a:.3g} / {n_a}; "
              f"within budget {np.mean(e_n <= budget):.3f}; stats {st}")
    print("theta sweep (median, interactions, theta):", sweep)
    for budget in (1e-6, 1e-5):
        med_n, n_n, st, e_n = rows[(budget, "network")]
        med_a, n_a, _, _ = rows[(budget, "analytic")]
        assert st["candidates"] > 0 and st["accepted"] > 0 and st["fallback"] < 0.05 * st["candidates"]
        assert med_n <= 1.05 * med_a and n_n <= 1.05 * n_a
        assert n_n < n_theta
        # fewer interactions than every theta of the sweep that is at least
        # as accurate (in time the wider theta wins on this walk: see above)
        assert all(n_n < n for med, n, _ in sweep if med <= med_n)
        assert np.mean(e_n <= budget) >= 0.95  # the bodies' errors within their budget
    assert rows[(1e-5, "network")][0] <= 1e-5


def test_simulate_learned_mode_matches_api(bh, tmp_path):
    """simulate --mode learned --model FILE (the reference's CLI, extended):
    a model saved with mlp_save drives the same steps as the C ABI with the
    same model, budget and criterion; 3 steps of 2,000 bodies, bit for bit."""
    import subprocess
    if not SIMULATE.exists():
        pytest.skip("simulate not built (run build())")
    feats, labels = [], []
    with _system(bh, 201, 60_000) as c:
        f, lab = c.learned_collect(THETA, 0.5, 3.0, G, max_pairs=800_000)
        ok = np.all(np.isfinite(f), axis=1) & np.isfinite(lab)
        feats.append(f[ok]); labels.append(lab[ok])
    params, scale, _ = bh.mlp_train(np.concatenate(feats), np.concatenate(labels), epochs=4, batch=2048, lr=2e-3,
                                    seed=0)
    model = tmp_path / "model.bhmlp"
    bh.mlp_save(model, params, scale)
    p2, s2 = bh.mlp_load(model)
    assert_bits_equal(p2, params, "saved parameters"); assert_bits_equal(s2, scale, "saved scaling")
    dump = tmp_path / "final.csv"
    r = subprocess.run([str(SIMULATE), "--generate", "2000", "--seed", "3", "--steps", "3", "--dt", "1h",
                        "--mode", "learned", "--model", str(model), "--budget", "1e-5", "--band", "0.5",
                        "--frac", "0.25", "--vs", "none", "--dump", str(dump)], capture_output=True, text=True,
                       cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Loaded 2000 bodies" in r.stdout
    pos, vel, mass, ids = bh.generate_system(3, 2000, 0.10, 0.0)
    with bh.Context(2000) as c:
        c.learned_set_model(params, scale, budget=1e-5, theta_max=3.0)
        c.learned_set_criterion(0.5, 0.25)
        c.set_bodies(pos, vel, mass, ids)
        c.step(DT, THETA, G, 3, bh.MODE_LEARNED, t=0.0)
        p, v, m, i, _ = c.get_bodies()
        c.compute_accelerations(THETA, G, 0.0, bh.MODE_LEARNED, download=False)
        stats = c.learned_stats()
    _, rmass, rpos, rvel = bh.read_csv(dump)
    rids = np.loadtxt(dump, delimiter=",", skiprows=1, usecols=0, dtype=np.uint64)
    assert_bits_equal(rids, i, "ids"); assert_bits_equal(rmass, m, "masses")
    assert_bits_equal(rpos, p, "positions"); assert_bits_equal(rvel, v, "velocities")
    assert stats["candidates"] > 0
    r = subprocess.run([str(SIMULATE), "--generate", "100", "--mode", "learned", "--vs", "none"],
                       capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 1 and "--model" in r.stderr


def test_step_graphs_follow_learned_parameters(bh):
    """Steps replayed from a captured graph take a changed budget, criterion
    and theta_max: 3 steps at one setting, then 3 at each of two others,
    with graphs on and off, bit for bit, and the settings change the
    interaction count.  (The analytic estimate alone decides at band 0, so
    an untrained network suffices.)"""
    rng = np.random.default_rng(5)
    params = he_params(rng)
    scale = np.concatenate([np.zeros(8, np.float32), np.ones(8, np.float32), np.full(8, -64.0, np.float32),
                            np.full(8, 64.0, np.float32), np.array([-6.0, 2.0], np.float32)])
    pos, vel, mass, ids = bh.generate_system(7, 20_000, 0.1, 0.05)
    settings = ((1e-7, 3.0, 0.0), (1e-4, 3.0, 0.0), (1e-4, 1.5, 0.0))
    runs = []
    for graphs in (True, False):
        with bh.Context(20_000) as c:
            c.set_step_graphs(graphs)
            c.set_bodies(pos, vel, mass, ids)
            counts = []
            for k, (budget, theta_max, band) in enumerate(settings):
                c.learned_set_model(params, scale, budget=budget, theta_max=theta_max)
                c.learned_set_criterion(band, 0.25)
                c.step(DT, THETA, G, 3, bh.MODE_LEARNED, t=0.0 if k == 0 else None)
                counts.append(c.interaction_count())
            runs.append((c.get_bodies()[:2], counts))
    (p_g, v_g), n_g = runs[0]
    (p_e, v_e), n_e = runs[1]
    assert_bits_equal(p_g, p_e, "positions"); assert_bits_equal(v_g, v_e, "velocities")
    assert n_g == n_e
    assert len(set(n_g)) == 3, n_g
