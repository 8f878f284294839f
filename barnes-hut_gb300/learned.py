"""Training of the learned acceptance criterion from seeded synthetic systems.

Pairs are collected by the engine's FP32 walk with the plain theta test and
labelled by the plain walk at theta_label (bh_learned_collect); the network is
trained by the engine's own GPU kernels (bh_mlp_train).  No reference
counterpart.
"""
from __future__ import annotations

import importlib

import numpy as np

bh = importlib.import_module("barnes-hut_gb300")


def collect_pairs(seeds, n_bodies, frac_outer=0.10, frac_trojan=0.05, theta=bh.THETA_DEFAULT, theta_label=0.5,
                  theta_max=3.0, max_pairs=10_000_000, G=bh.G_DEFAULT):
    """(features (k, 8), labels (k,)) from one system per seed, at most
    max_pairs in total (an even share per seed)."""
    per = max(1, max_pairs // max(1, len(seeds)))
    feats, labels = [], []
    with bh.Context(n_bodies) as c:
        for s in seeds:
            pos, vel, mass, ids = bh.generate_system(int(s), n_bodies, frac_outer, frac_trojan)
            c.set_bodies(pos, vel, mass, ids)
            c.compute_bbox(); c.compute_keys(); c.sort_bodies(); c.build_tree()
            f, l = c.learned_collect(theta, theta_label, theta_max, G, max_pairs=per)
            ok = np.all(np.isfinite(f), axis=1) & np.isfinite(l)
            feats.append(f[ok]); labels.append(l[ok])
    return np.concatenate(feats), np.concatenate(labels)


def train(seeds, n_bodies, epochs=10, batch=4096, lr=2e-3, seed=0, **collect_kw):
    """Collects pairs and trains; returns (params, scale, losses, n_pairs)."""
    F, L = collect_pairs(seeds, n_bodies, **collect_kw)
    params, scale, losses = bh.mlp_train(F, L, epochs=epochs, batch=batch, lr=lr, seed=seed)
    return params, scale, losses, len(L)
