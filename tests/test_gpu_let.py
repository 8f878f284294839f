"""Locally essential tree export (createInteractionListForRank,
src/exchange.cpp:117-179) on the GPU: bit-exact against the compiled
reference's exports (golden fixtures), against the oracle on larger systems,
and at 4M bodies through properties that characterise the exported set."""
from __future__ import annotations

import hashlib

import numpy as np
import pytest

from conftest import assert_bits_equal

pytestmark = pytest.mark.gpu


def _local_ctx(bh, pos, vel, mass, ids, bb):
    """A context holding the local bodies, keys in the global box, and the
    tree of buildOctreeBottomUp without the merge (what main.cpp exports)."""
    c = bh.Context(max(len(mass), 1))
    c.set_bodies(pos, vel, mass, ids)
    if len(mass):
        c.set_bbox(bb)
        c.compute_keys()
        c.sort_bodies()
        c.build_tree(merge=False)
    return c


def _sorted(p, d, m, com):
    o = np.lexsort((p, d))
    return p[o], d[o], m[o], np.ascontiguousarray(com[o])


def _digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


@pytest.mark.parametrize("system", ["synthetic_1000", "synthetic_19054"])
def test_let_export_matches_reference_golden(bh, golden, system):
    g = golden(f"{system}.npz")
    f = golden("let_export.npz")
    bb = f[f"{system}/bbox"]
    n = len(g["mass"])
    for ci in range(int(f[f"{system}/n_cases"][0])):
        c = f"{system}/c{ci}/"
        sel = np.nonzero(np.unpackbits(f[c + "local"])[:n].astype(bool))[0]
        with _local_ctx(bh, g["pos"][sel], g["vel"][sel], g["mass"][sel], g["ids"][sel], bb) as ctx:
            out = ctx.let_export(f[c + "boxes"], bb, float(f[c + "theta2"][0]), int(f[c + "max_depth"][0]))
        p, d, m, com = _sorted(*out)
        assert len(p) == int(f[c + "count"][0]), ci
        assert np.array_equal(np.bincount(d, minlength=22), f[c + "depth_hist"]), ci
        assert _digest(p, d, m, com) == str(f[c + "digest"][0]), ci
        if c + "prefix" in f:
            assert_bits_equal(p, f[c + "prefix"], f"case {ci} prefixes")
            assert_bits_equal(d, f[c + "depth"], f"case {ci} depths")
            assert_bits_equal(m, f[c + "mass"], f"case {ci} masses")
            assert_bits_equal(com, f[c + "com"], f"case {ci} centres of mass")


def _bucket_domains(keys, bucket_bits, nranks):
    """update_rank_domains' split (src/load_balancing.cpp:12-65): per rank
    the owner of each body and the non-empty bucket prefixes."""
    bidx = (keys >> np.uint64(63 - bucket_bits)).astype(np.int64)
    hist = np.bincount(bidx, minlength=1 << bucket_bits)
    ideal = (len(keys) + nranks - 1) // nranks
    split, run = [], 0
    for i, h in enumerate(hist.tolist()):
        run += h
        if len(split) < nranks - 1 and run >= (len(split) + 1) * ideal:
            split.append(i)
    owner = np.searchsorted(np.array(split, np.int64), np.arange(1 << bucket_bits), side="right")
    body_owner = owner[bidx]
    doms = [(np.nonzero((hist > 0) & (owner == r))[0].astype(np.uint64)) << np.uint64(63 - bucket_bits)
            for r in range(nranks)]
    return body_owner, doms


def test_let_export_matches_oracle_200k(bh, port):
    """200,000 bodies split over 4 ranks by 18-bit buckets (the reference's
    default): rank 0's export to each other rank equals the oracle's."""
    pos, vel, mass, ids = bh.generate_system(31, 200_000, 0.1, 0.05)
    bb = port.bbox(pos)
    keys = port.keys(pos, bb)
    owner, doms = _bucket_domains(keys, 18, 4)
    sel = np.nonzero(owner == 0)[0]
    sk, sp, sm, _, _, _ = port.sort(keys[sel], pos[sel], mass[sel], vel[sel], ids[sel])
    tree = port.tree(sk, sp, sm, merge=False)
    with _local_ctx(bh, pos[sel], vel[sel], mass[sel], ids[sel], bb) as ctx:
        for r, (theta, md) in zip(range(1, 4), ((1.05, 21), (0.6, 21), (1.05, 9))):
            boxes = bh.let_bucket_boxes(doms[r], 18, bb)
            got = _sorted(*ctx.let_export(boxes, bb, theta * theta, md))
            want = port.let_export(tree, boxes, bb, theta * theta, md)
            assert len(got[0]) == len(want[0]) > 0, r
            for a, b, what in zip(got, want, ("prefix", "depth", "mass", "com")):
                assert_bits_equal(a, b, f"rank {r} {what}")
    tree.close()


def _cell_boxes(prefix, depth, bb):
    """getBoundingBoxForCell (src/bounding_box.cpp:55-75) in numpy float64."""
    lo = np.empty((len(prefix), 3)); hi = np.empty((len(prefix), 3))
    d = depth.astype(np.int64)
    bits = np.where(d > 0, prefix >> (63 - 3 * d).clip(0, 63).astype(np.uint64), 0).astype(np.uint64)
    scale = 1.0 / (2.0 ** d)
    for a in range(3):
        v = np.zeros(len(prefix), np.uint64)
        for b in range(21):
            v |= np.where(b < d, ((bits >> np.uint64(3 * b + a)) & np.uint64(1)) << np.uint64(b), 0).astype(np.uint64)
        span = bb[3 + a] - bb[a]
        lo[:, a] = bb[a] + (v.astype(np.float64) * scale) * span
        hi[:, a] = lo[:, a] + span / (2.0 ** d)
    return lo, hi


def _opens(lo, hi, boxes, theta2):
    """Whether each cell fails the opening test against any box."""
    s = hi[:, 0] - lo[:, 0]
    for a in (1, 2):
        t = hi[:, a] - lo[:, a]
        s = np.where(s < t, t, s)
    s2 = s * s
    out = np.zeros(len(lo), bool)
    for b in boxes:
        e = []
        for a in range(3):
            x = lo[:, a] - b[3 + a]; y = b[a] - hi[:, a]
            m = np.where(x < y, y, x)
            e.append(np.where(0.0 < m, m, 0.0))
        d2 = (e[0] * e[0] + e[1] * e[1]) + e[2] * e[2]
        out |= s2 >= theta2 * d2
    return out


def test_let_export_box_order_and_scale(bh, port):
    """The group prefilter of the export against the oracle where its groups
    are loose or it is off: the other ranks' bucket boxes in shuffled order
    (hulls of scattered boxes), 3,000 random boxes, and the same system and
    boxes scaled by 1e13 (coordinates beyond 2^40, where every box test is
    FP64)."""
    pos0, vel, mass, ids = bh.generate_system(33, 60_000, 0.1, 0.05)
    rng = np.random.default_rng(34)
    for scale in (1.0, 1e13):
        pos = pos0 * scale
        bb = port.bbox(pos)
        keys = port.keys(pos, bb)
        owner, doms = _bucket_domains(keys, 18, 4)
        sel = np.nonzero(owner == 0)[0]
        sk, sp, sm, _, _, _ = port.sort(keys[sel], pos[sel], mass[sel], vel[sel], ids[sel])
        tree = port.tree(sk, sp, sm, merge=False)
        lo, hi = bb[:3], bb[3:]
        c = rng.uniform(lo, hi, (3000, 3))
        h = rng.uniform(0.0, 0.02, (3000, 3)) * (hi - lo)
        random_boxes = np.concatenate([c - h, c + h], axis=1)
        with _local_ctx(bh, pos[sel], vel[sel], mass[sel], ids[sel], bb) as ctx:
            for r in (1, 2, 3):
                boxes = bh.let_bucket_boxes(doms[r], 18, bb)
                for name, bx in (("bucket order", boxes), ("shuffled", boxes[rng.permutation(len(boxes))]),
                                 ("random", random_boxes)):
                    for theta in (0.7, 1.05):
                        got = _sorted(*ctx.let_export(bx, bb, theta * theta, 21))
                        want = port.let_export(tree, bx, bb, theta * theta, 21)
                        assert len(got[0]) == len(want[0]) > 0, (scale, r, name, theta)
                        for a, b, what in zip(got, want, ("prefix", "depth", "mass", "com")):
                            assert_bits_equal(a, b, f"scale {scale} rank {r} {name} theta {theta}: {what}")
        tree.close()


def test_let_export_properties_4m(bh):
    """4,000,000 bodies, rank 0 of 8 (18-bit buckets) exporting to rank 1
    at theta 0.7:
    the kept cells tile rank 0's keys (every body lies in exactly one kept
    cell), every kept cell above max_depth passes the opening test against
    every box, and the parent of every kept cell fails it for some box --
    which together determine the reference's exported set."""
    n = 4_000_000
    pos, vel, mass, ids = bh.generate_system(32, n, 0.1, 0.05)
    with bh.Context(n) as full:
        full.set_bodies(pos, vel, mass, ids)
        bb = full.compute_bbox()
        keys = full.compute_keys()
    owner, doms = _bucket_domains(keys, 18, 8)
    sel = np.nonzero(owner == 0)[0]
    theta2 = 0.7 ** 2
    boxes = bh.let_bucket_boxes(doms[1], 18, bb)
    with _local_ctx(bh, pos[sel], vel[sel], mass[sel], ids[sel], bb) as ctx:
        p, d, m, com = _sorted(*ctx.let_export(boxes, bb, theta2, 21))
        lkeys = np.sort(ctx.compute_keys())
    assert 0 < len(p) < len(sel)
    # tiling of rank 0's keys
    o = np.argsort(p, kind="stable")
    start = p[o]; width = np.uint64(1) << (np.uint64(63) - np.uint64(3) * d[o].astype(np.uint64))
    end = start + width  # exclusive; no overflow below 2^63
    assert np.all(start[1:] >= end[:-1]), "kept cells overlap"
    j = np.searchsorted(start, lkeys, side="right") - 1
    assert np.all(j >= 0) and np.all(lkeys < end[j]), "a body lies in no kept cell"
    # the kept cells carry rank 0's whole mass
    assert np.isclose(m.sum(), mass[sel].sum(), rtol=1e-12)
    # the opening test decides each kept cell and each parent
    lo, hi = _cell_boxes(p, d, bb)
    assert not np.any(_opens(lo, hi, boxes, theta2)[d < 21]), "a kept cell fails the test"
    dp = d.astype(np.int64) - 1
    par = d > 0
    mask = np.where(dp[par] > 0, (~np.uint64(0)) << (63 - 3 * dp[par]).clip(0, 63).astype(np.uint64), 0)
    pp = (p[par] & mask.astype(np.uint64)).astype(np.uint64)
    plo, phi = _cell_boxes(pp, dp[par].astype(np.uint8), bb)
    assert np.all(_opens(plo, phi, boxes, theta2)), "a kept cell's parent passes the test"


def test_pseudo_leaf_tree_matches_reference_golden(bh, golden):
    """buildTreeFromPseudoLeaves on the device against the compiled
    reference: the same cells; sums within 1e-14 relative (the reference adds
    children in hash-map order, the device in octant order)."""
    f = golden("pseudo_tree.npz")
    with bh.Context(16) as ctx:
        p, d, m, c = ctx.pseudo_leaf_tree(f["prefix"], f["depth"], f["mass"], f["com"])
    assert_bits_equal(p, f["tree_prefix"], "prefixes")
    assert_bits_equal(d, f["tree_depth"], "depths")
    assert np.all(np.abs(m - f["tree_mass"]) <= 1e-14 * np.abs(f["tree_mass"]))
    scale = np.abs(f["tree_com"]).max(axis=1, keepdims=True)
    assert np.all(np.abs(c - f["tree_com"]) <= 1e-14 * scale)


def test_pseudo_leaf_tree_matches_oracle_bits(bh, port):
    """The LETs that rank 0 of an 8-way split of 1,000,000 bodies receives
    from the other seven ranks (exported on the device), built into a map on
    the device and by the oracle, which sums children in the same octant
    order: bit for bit.  Empty input and all-invalid input give no cells."""
    n = 1_000_000
    pos, vel, mass, ids = bh.generate_system(33, n, 0.1, 0.05)
    with bh.Context(n) as full:
        full.set_bodies(pos, vel, mass, ids)
        bb = full.compute_bbox()
        keys = full.compute_keys()
    owner, doms = _bucket_domains(keys, 18, 8)
    boxes0 = bh.let_bucket_boxes(doms[0], 18, bb)
    parts = []
    for r in range(1, 8):
        sel = np.nonzero(owner == r)[0]
        with _local_ctx(bh, pos[sel], vel[sel], mass[sel], ids[sel], bb) as ctx:
            parts.append(ctx.let_export(boxes0, bb, 0.6 ** 2, 21))
    p = np.concatenate([x[0] for x in parts]); d = np.concatenate([x[1] for x in parts])
    m = np.concatenate([x[2] for x in parts]); c = np.concatenate([x[3] for x in parts])
    assert len(p) > 10_000
    with bh.Context(16) as ctx:
        got = ctx.pseudo_leaf_tree(p, d, m, c)
        empty = ctx.pseudo_leaf_tree(p[:0], d[:0], m[:0], c[:0])
        bad = ctx.pseudo_leaf_tree(p[:3], d[:3], np.array([0.0, np.nan, -1.0]), c[:3])
    t = port.pseudo_tree(p, d, m, c)
    want = t.records()
    t.close()
    for a, b, what in zip(got, want, ("prefix", "depth", "mass", "com")):
        assert_bits_equal(a, b, what)
    assert len(empty[0]) == 0 and len(bad[0]) == 0


def test_let_forces_match_reference_golden(bh, golden):
    """computeAccelerationsWithLET and ...WithRemoteDirectSum on the device
    against the compiled reference (rank 0 of a 4-way split of the 1,000-body
    system): within 1e-13 relative."""
    f = golden("pseudo_tree.npz")
    g = golden("synthetic_1000.npz")
    nv = int(f["n_valid"][0])
    sel = np.nonzero(np.unpackbits(f["local"])[:len(g["mass"])].astype(bool))[0]
    with _local_ctx(bh, g["pos"][sel], g["vel"][sel], g["mass"][sel], g["ids"][sel], f["bbox"]) as ctx:
        rec = (f["prefix"], f["depth"], f["mass"], f["com"])
        valid = tuple(a[:nv] for a in rec)
        got = {"let_acc": ctx.let_accelerations(*valid, theta=1.05),
               "let_acc_all": ctx.let_accelerations(*rec, theta=1.05),
               "letds_acc": ctx.let_accelerations(*valid, theta=1.05, direct=True)}
    for k, a in got.items():
        want = f[k]
        rel = np.linalg.norm(a - want, axis=1) / np.linalg.norm(want, axis=1)
        assert rel.max() <= 1e-13, k


def test_let_forces_match_oracle_bits(bh, port):
    """300,000 bodies over 4 ranks (9-bit buckets): rank 0's forces with the
    records the other ranks export to it, on the device and in the oracle
    (which builds the pseudo-leaf map in the same octant order and sums the
    records in the same order): bit for bit, both LET forms; the local tree
    is unchanged afterwards."""
    n = 300_000
    pos, vel, mass, ids = bh.generate_system(34, n, 0.1, 0.05)
    bb = port.bbox(pos)
    keys = port.keys(pos, bb)
    owner, doms = _bucket_domains(keys, 9, 4)
    boxes0 = bh.let_bucket_boxes(doms[0], 9, bb)
    parts = []
    for r in range(1, 4):
        sel = np.nonzero(owner == r)[0]
        with _local_ctx(bh, pos[sel], vel[sel], mass[sel], ids[sel], bb) as ctx:
            parts.append(ctx.let_export(boxes0, bb, 1.05 ** 2, 21))
    rec = tuple(np.concatenate([x[k] for x in parts]) for k in range(4))
    sel = np.nonzero(owner == 0)[0]
    sk, sp, sm, _, _, _ = port.sort(keys[sel], pos[sel], mass[sel], vel[sel], ids[sel])
    tree = port.tree(sk, sp, sm, merge=False)
    want = [port.let_accelerations(tree, rec, sk, sp, 1.05, 1.48812e-34, bb, direct=d) for d in (False, True)]
    tree.close()
    with _local_ctx(bh, pos[sel], vel[sel], mass[sel], ids[sel], bb) as ctx:
        before = ctx.export_tree()
        got = [ctx.let_accelerations(*rec, theta=1.05, direct=d) for d in (False, True)]
        after = ctx.export_tree()
        plain = ctx.compute_accelerations(1.05)
    assert len(rec[0]) > 1000
    assert_bits_equal(got[0], want[0], "LET forces")
    assert_bits_equal(got[1], want[1], "LET remote direct sum forces")
    for a, b in zip(before, after):
        assert_bits_equal(a, b, "local tree")
    # the imported records move the forces by about the remote share
    assert np.median(np.linalg.norm(got[0] - plain, axis=1) / np.linalg.norm(plain, axis=1)) > 1e-9


def test_let_edge_cases_match_oracle(bh, port):
    """Small and degenerate inputs against the oracle: one body, two bodies
    with one key, max_depth 0 and 1, no boxes, a box around everything,
    records at depth 0 and at depth 21, a record with zero mass."""
    rng = np.random.default_rng(5)
    systems = {
        "one": (np.array([[0.5, -0.25, 0.125]]), np.array([2.0e20])),
        "two_same_key": (np.array([[1.0, 1.0, 1.0], [1.0, 1.0, 1.0 + 1e-15], [-3.0, 2.0, 0.5]]),
                         np.array([1e18, 2e18, 3e18])),
        "cluster": (rng.normal(0, 1, (500, 3)), rng.uniform(1e15, 1e20, 500)),
    }
    for name, (pos, mass) in systems.items():
        n = len(mass)
        vel = np.zeros((n, 3)); ids = np.arange(n, dtype=np.uint64)
        bb = port.bbox(pos) if n > 1 else np.array([0.0, -1.0, -1.0, 1.0, 1.0, 1.0])
        keys = port.keys(pos, bb)
        sk, sp, sm, _, _, _ = port.sort(keys, pos, mass, vel, ids)
        tree = port.tree(sk, sp, sm, merge=False)
        # boxes at exactly one root side from the root cell and from a
        # depth-3 cell (ties of s^2 >= theta^2 d^2 at theta = 1, decided by
        # the FP64 test behind the FP32 prescreen)
        side = max(bb[3] - bb[0], bb[4] - bb[1], bb[5] - bb[2])
        tie = np.array([[bb[3] + side, bb[1], bb[2], bb[3] + 2 * side, bb[4], bb[5]],
                        [bb[0], bb[1], bb[2] - side / 8 - (bb[5] - bb[2]) / 8, bb[3], bb[4], bb[2] - side / 8]])
        box_sets = [np.array([[5.0, 5.0, 5.0, 6.0, 6.0, 6.0]]), np.array([[-9.0, -9.0, -9.0, 9.0, 9.0, 9.0]]),
                    np.zeros((0, 6)), tie]
        with _local_ctx(bh, pos, vel, mass, ids, bb) as ctx:
            for boxes in box_sets:
                for theta, md in ((1.05, 21), (0.3, 0), (0.3, 1), (2.0, 25), (1.0, 21)):
                    got = _sorted(*ctx.let_export(boxes, bb, theta * theta, md))
                    want = port.let_export(tree, boxes, bb, theta * theta, md)
                    for a, b, what in zip(got, want, ("prefix", "depth", "mass", "com")):
                        assert_bits_equal(a, b, f"{name} {len(boxes)} boxes theta {theta} max_depth {md}: {what}")
            recs = [
                (np.array([0], np.uint64), np.array([0], np.uint8), np.array([5e19]), np.array([[3.0, 3.0, 3.0]])),
                (np.array([sk[0]], np.uint64), np.array([21], np.uint8), np.array([1e19]), sp[:1] + 1e-3),
                (np.array([0, sk[-1]], np.uint64), np.array([0, 21], np.uint8), np.array([0.0, 4e19]),
                 np.array([[1.0, 1.0, 1.0], [-1.0, 0.0, 2.0]])),
            ]
            for r in recs:
                t = port.pseudo_tree(*r)
                want_map = t.records()
                t.close()
                got_map = ctx.pseudo_leaf_tree(*r)
                for a, b, what in zip(got_map, want_map, ("prefix", "depth", "mass", "com")):
                    assert_bits_equal(a, b, f"{name} pseudo map {what}")
                for direct in (False, True):
                    got = ctx.let_accelerations(*r, theta=1.05, direct=direct)
                    want = port.let_accelerations(tree, r, sk, sp, 1.05, 1.48812e-34, bb, direct=direct)
                    assert_bits_equal(got, want, f"{name} LET forces direct={direct}")
        tree.close()
