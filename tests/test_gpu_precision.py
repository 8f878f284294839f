"""The FP32 far-field precision form (BH_MODE_FP32_FAR): accelerations measured
against the FP64 direct-sum sampler, and against the plain FP64 mode."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import DT, G, THETA

pytestmark = pytest.mark.gpu


def rel_err(a, ref):
    return np.linalg.norm(a - ref, axis=1) / np.linalg.norm(ref, axis=1)


@pytest.fixture(scope="module")
def system(bh):
    pos, vel, mass, ids = bh.generate_system(11, 300_149, 0.1, 0.0)
    ctx = bh.Context(len(mass))
    ctx.set_bodies(pos, vel, mass, ids)
    ctx.compute_bbox(); ctx.compute_keys(); ctx.sort_bodies(); ctx.build_tree()
    rng = np.random.default_rng(1)
    sample = np.sort(rng.choice(len(mass), 2048, replace=False))
    sample = np.unique(np.concatenate([sample, np.arange(9)]))  # include the Sun and planets' slots
    ref = ctx.direct_sum(sample, G)
    yield ctx, sample, ref
    ctx.close()


@pytest.mark.parametrize("theta", [0.5, 0.8, 1.05])
def test_fp32_far_error_vs_direct_sum(bh, system, theta):
    ctx, sample, ref = system
    a32 = ctx.compute_accelerations(theta, G, 0.0, bh.MODE_FP32_FAR)
    a64 = ctx.compute_accelerations(theta, G, 0.0, bh.MODE_PLAIN_FP64)
    e32 = rel_err(a32[sample], ref)
    e64 = rel_err(a64[sample], ref)
    # Tolerance: the metric's budget, median relative error <= 1e-5.
    assert np.median(e32) <= 1e-5
    assert np.all(np.isfinite(a32))
    # The group acceptance is at least as strict as the per-body test, and
    # the dominant Sun/planet terms are exact FP64, so the FP32 form is not
    # less accurate than the plain FP64 form beyond FP32 rounding.
    assert np.median(e32) <= np.median(e64) + 1e-6
    assert np.quantile(e32, 0.99) <= max(1e-4, 2 * np.quantile(e64, 0.99))


def test_fp32_far_tree_rebuild_restores_reference_tree(bh, system, golden):
    ctx, _, _ = system
    ctx.compute_accelerations(THETA, G, 0.0, bh.MODE_FP32_FAR)
    # export always reports the reference's tree (real masses)
    prefix, depth, mass, com = ctx.export_tree()
    assert depth[0] == 0 and mass[0] > 1.9e30  # the root holds the Sun again


def test_fp32_far_trajectory_close_to_fp64(bh):
    pos, vel, mass, ids = bh.generate_system(12, 50_000, 0.1, 0.05)
    out = {}
    for mode in (bh.MODE_PLAIN_FP64, bh.MODE_FP32_FAR):
        with bh.Context(len(mass)) as c:
            c.set_bodies(pos, vel, mass, ids)
            c.step(DT, THETA, G, nsteps=20, mode=mode, t=0.0)
            p, v, m, i, a = c.get_bodies()
            o = np.argsort(i)
            out[mode] = (p[o], v[o])
    dp = np.abs(out[0][0] - out[2][0]).max()
    assert dp < 1e-9  # AU after 20 one-hour steps


def test_direct_bodies_summed_exactly(bh):
    """Nine massive bodies only: no far field at all, FP64 direct sums."""
    pos, vel, mass, ids = bh.generate_system(3, 9, 0.0, 0.0)
    with bh.Context(9) as c:
        c.set_bodies(pos, vel, mass, ids)
        c.compute_bbox(); c.compute_keys(); c.sort_bodies(); c.build_tree()
        a = c.compute_accelerations(THETA, G, 0.0, bh.MODE_FP32_FAR)
        ref = c.direct_sum(np.arange(9), G)
    assert np.all(rel_err(a, ref) < 1e-14)


def test_fp32_far_interaction_set_tracks_per_body_theta(bh, system, port):
    """The FP32 walk applies each body's own theta test on the far-field tree
    (the direct bodies' masses removed, which moves the centres of mass of
    the cells around them, and the direct terms counted instead of the
    direct bodies' leaves): the total stays within 15 % of the FP64 walk's."""
    ctx, _, _ = system
    ctx.compute_accelerations(THETA, G, 0.0, bh.MODE_FP64_LIST)
    c64 = ctx.interaction_counts().astype(np.int64)
    ctx.compute_accelerations(THETA, G, 0.0, bh.MODE_FP32_FAR)
    c32 = ctx.interaction_counts().astype(np.int64)
    assert np.all(c32 > 0)
    assert abs(c32.sum() / c64.sum() - 1) < 0.15


@pytest.mark.parametrize("theta", [0.8, 1.05, 1.6])
def test_fp32_group_refines_each_bodys_own_set(bh, system, theta):
    """BH_MODE_FP32_GROUP accepts a node for the whole warp group only when
    every body's own test accepts it: each body's interaction set is then
    its own set or a refinement of it, so its count is never lower than in
    BH_MODE_FP32_FAR at the same theta, and its error against the FP64
    direct sum is no higher in the median (tolerance: FP32 rounding, 2e-8)."""
    ctx, sample, ref = system
    a_b = ctx.compute_accelerations(theta, G, 0.0, bh.MODE_FP32_FAR)
    c_b = ctx.interaction_counts().astype(np.int64)
    a_g = ctx.compute_accelerations(theta, G, 0.0, bh.MODE_FP32_GROUP)
    c_g = ctx.interaction_counts().astype(np.int64)
    assert np.all(np.isfinite(a_g))
    assert np.all(c_g >= c_b)
    assert c_g.sum() > c_b.sum()
    assert ctx.interaction_count() == c_g.sum()
    e_b, e_g = rel_err(a_b[sample], ref), rel_err(a_g[sample], ref)
    assert np.median(e_g) <= np.median(e_b) + 2e-8
    assert np.median(e_g) <= 1e-5


def test_fp32_group_steps_match_single_launches(bh):
    """The group form through bh_step (graph replays) equals the kernels
    launched one by one, and its trajectory stays with the FP64 form's."""
    pos, vel, mass, ids = bh.generate_system(13, 20_000, 0.1, 0.05)
    out = {}
    for graphs in (True, False):
        with bh.Context(len(mass)) as c:
            c.set_step_graphs(graphs)
            c.set_bodies(pos, vel, mass, ids)
            c.step(DT, THETA, G, nsteps=6, mode=bh.MODE_FP32_GROUP, t=0.0)
            out[graphs] = c.get_bodies()
    for a, b in zip(out[True], out[False]):
        assert np.array_equal(a, b)
    with bh.Context(len(mass)) as c:
        c.set_bodies(pos, vel, mass, ids)
        c.step(DT, THETA, G, nsteps=6, mode=bh.MODE_PLAIN_FP64, t=0.0)
        p64, _, _, i64, _ = c.get_bodies()
    p, _, _, i, _ = out[True]
    assert np.abs(p[np.argsort(i)] - p64[np.argsort(i64)]).max() < 1e-10


def test_fp32_steps_then_record_readers(bh):
    """An FP32 step builds only the FP32 walk's node records; the calls that
    read the FP64 ones (invariants through the tree, the tree export, the
    learned criterion's pair collection) write them first, and see what a
    fresh build of the same state gives."""
    pos, vel, mass, ids = bh.generate_system(23, 40_000, 0.1, 0.05)
    n = len(mass)
    with bh.Context(n) as c:
        c.set_bodies(pos, vel, mass, ids)
        c.step(DT, THETA, G, nsteps=3, mode=bh.MODE_FP32_GROUP, t=0.0)
        inv1 = c.invariants(G, THETA)
        exp1 = c.export_tree()
        p, v, m, i, _ = c.get_bodies()
        c.step(DT, THETA, G, nsteps=1, mode=bh.MODE_FP32_FAR, t=1.0)
        f1, l1 = c.learned_collect(THETA, 0.5, 3.0, G, max_pairs=3_000_000)
        state = c.get_bodies()
    with bh.Context(n) as c2:
        c2.set_bodies(p, v, m, i)
        c2.compute_bbox(); c2.compute_keys(); c2.sort_bodies(); c2.build_tree()
        inv2 = c2.invariants(G, THETA)
        exp2 = c2.export_tree()
        c2.set_bodies(*state[:4])
        c2.compute_bbox(); c2.compute_keys(); c2.sort_bodies(); c2.build_tree()
        f2, l2 = c2.learned_collect(THETA, 0.5, 3.0, G, max_pairs=3_000_000)
    for a, b in zip(exp1, exp2):
        assert np.array_equal(a, b)
    for k in ("E", "K", "U"):
        assert abs(inv1[k] - inv2[k]) <= 1e-12 * abs(inv2[k])
    # the pairs come out in the order the warps reach them: compare as sets
    assert 0 < len(l1) == len(l2) < 3_000_000
    assert np.allclose(np.sort(l1), np.sort(l2), rtol=0, atol=1e-3)
    assert np.allclose(np.sort(f1, axis=0), np.sort(f2, axis=0), rtol=0, atol=1e-4)


def test_second_moment_spread_matches_fp64(bh):
    """The second-moment pass (learned features): per device node,
    sqrt(Q/m) of the far-field masses, Q = sum m |x - com|^2 over the
    node's bodies, against an FP64 sum over the same bodies (the FP32
    result: 1e-5 relative)."""
    pos, vel, mass, ids = bh.generate_system(31, 3000, 0.1, 0.05)
    with bh.Context(3000) as c:
        c.set_bodies(pos, vel, mass, ids)
        c.compute_bbox(); keys = c.compute_keys(); c.sort_bodies(); c.build_tree()
        prefix, depth = c.tree_slots()
        spread = c.tree_spread()
        p, _, m, i, _ = c.get_bodies()
    sk = np.sort(keys, kind="stable")
    mf = np.where(i < 9, 0.0, m)
    checked = 0
    for s in range(len(prefix)):
        d = int(depth[s])
        lo = np.searchsorted(sk, prefix[s], side="left")
        hi = np.searchsorted(sk, prefix[s] + (np.uint64(1) << np.uint64(63 - 3 * d)), side="left") \
            if d > 0 else len(sk)
        w = mf[lo:hi]
        M = w.sum()
        if M == 0:
            assert spread[s] == 0.0
            continue
        com = (w[:, None] * p[lo:hi]).sum(axis=0) / M
        q = (w * ((p[lo:hi] - com) ** 2).sum(axis=1)).sum()
        ref = np.sqrt(q / M)
        assert abs(spread[s] - ref) <= 1e-5 * ref + 1e-12 * np.abs(com).max(), (s, d, spread[s], ref)
        checked += 1
    assert checked > 2000


def test_kepler_batch_on_gpu_matches_host(bh):
    """The batched GPU conversion of orbital elements agrees with the host
    restatement of convertKeplerToCartesian to 1e-12 relative (the two math
    libraries round sin, cos and atan2 differently in the last bits), on
    asteroid-belt elements, and is faster than the host at 1M bodies."""
    import time
    rng = np.random.default_rng(9)
    n = 1_000_000
    mu = 1.48812e-34 * 1.989e30
    el = np.stack([rng.uniform(0, 0.3, n), rng.uniform(2.1, 3.3, n), rng.uniform(0, 0.35, n),
                   rng.uniform(0, 2 * np.pi, n), rng.uniform(0, 2 * np.pi, n), rng.uniform(0, 2 * np.pi, n),
                   np.full(n, 2451544.5), np.full(n, mu)], axis=1)
    t0 = time.perf_counter(); host = bh.kepler_to_cartesian(el); t1 = time.perf_counter()
    bh.kepler_to_cartesian_gpu(el[:1000])  # context set-up outside the timing
    t2 = time.perf_counter(); dev = bh.kepler_to_cartesian_gpu(el); t3 = time.perf_counter()
    print(f"host {t1 - t0:.3f} s, gpu {t3 - t2:.3f} s for {n} bodies")
    for sl in (slice(0, 3), slice(3, 6)):
        d = np.linalg.norm(dev[:, sl] - host[:, sl], axis=1) / np.linalg.norm(host[:, sl], axis=1)
        assert d.max() < 1e-12
    assert t3 - t2 < t1 - t0
