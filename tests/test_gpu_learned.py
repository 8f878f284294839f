"""The learned acceptance criterion: the GPU's own forward/backward kernels
against the FP64 CPU restatement, the traversal's fused (mma.sync) inference
against the same, and the end-to-end pipeline -- pairs labelled by the plain
walk at theta = 0.5, training on the GPU, and what the trained network gains
over the theta criterion without it, measured against the FP64 direct sum."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import G, THETA

pytestmark = pytest.mark.gpu


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


def test_learned_pipeline_gains_over_theta(bh):
    feats, labels = [], []
    for seed in (101, 102, 103):
        with _system(bh, seed, 60_000) as c:
            f, l = c.learned_collect(THETA, 0.5, 3.0, G, max_pairs=1_500_000)
            ok = np.all(np.isfinite(f), axis=1) & np.isfinite(l)
            feats.append(f[ok]); labels.append(l[ok])
    F = np.concatenate(feats); L = np.concatenate(labels)
    assert len(L) > 50_000
    params, scale, losses = bh.mlp_train(F, L, epochs=8, batch=2048, lr=2e-3, seed=0)
    # standardised MSE (1.0 = predicting the mean): the network learns the labels
    assert losses[-1] < 0.3 and losses[-1] < losses[0]
    # unseen system: theta criterion alone vs learned criterion at budget 1e-5
    with _system(bh, 104, 60_000) as c:
        rng = np.random.default_rng(2)
        sample = np.sort(rng.choice(c.n, 1024, replace=False))
        ref = c.direct_sum(sample, G)
        a_theta = c.compute_accelerations(THETA, G, 0.0, bh.MODE_FP32_FAR)
        n_theta = c.interaction_count()
        c.learned_set_model(params, scale, budget=1e-6, theta_max=3.0)
        a_learn = c.compute_accelerations(THETA, G, 0.0, bh.MODE_LEARNED)
        n_learn = c.interaction_count()
        stats = c.learned_stats()
    e_theta = np.linalg.norm(a_theta[sample] - ref, axis=1) / np.linalg.norm(ref, axis=1)
    e_learn = np.linalg.norm(a_learn[sample] - ref, axis=1) / np.linalg.norm(ref, axis=1)
    print(f"theta: {n_theta} interactions, median err {np.median(e_theta):.3g}; learned: {n_learn} "
          f"interactions, median err {np.median(e_learn):.3g}; stats {stats}")
    assert stats["candidates"] > 0 and stats["accepted"] > 0
    assert stats["fallback"] < 0.5 * stats["candidates"]
    assert n_learn < n_theta          # the gain: fewer interactions ...
    assert np.median(e_learn) <= 1e-5  # ... within the metric's error budget
