"""Pins the oracle (the C restatement of the reference's path) to the golden
fixtures that the reference's own compiled sources produced, and -- where the
reference checkout is present -- directly to the compiled reference."""
from __future__ import annotations

import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from conftest import DT, G, GOLDEN, THETA, assert_bits_equal

EDGE = ["one", "two", "duplicate_key", "coplanar", "single_point", "massless", "massive"]


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def run_stages(o, pos, vel, mass, ids, theta=THETA):
    bb = o.bbox(pos)
    keys = o.keys(pos, bb)
    sk, sp, sm, sv, si, _ = o.sort(keys, pos, mass, vel, ids)
    tree = o.tree(sk, sp, sm)
    rec = tree.records()
    acc = o.accelerations(tree, sk, sp, theta, G, 0.0, bb)
    tree.close()
    return bb, keys, (sk, sp, sm, sv, si), rec, acc


@pytest.mark.parametrize("case", EDGE)
def test_edge_cases_bit_exact(port, golden, case):
    g = golden("edge_cases.npz")
    pos, vel, mass, ids = (g[f"{case}/{k}"] for k in ("pos", "vel", "mass", "ids"))
    bb, keys, srt, rec, acc = run_stages(port, pos, vel, mass, ids)
    assert_bits_equal(bb, g[f"{case}/bbox"], "bbox")
    assert_bits_equal(keys, g[f"{case}/keys"], "keys")
    for got, name in zip(srt, ("sorted_keys", "sorted_pos", "sorted_mass", "sorted_vel", "sorted_ids")):
        if case == "duplicate_key" and name != "sorted_keys":
            continue  # tie order of std::sort is unspecified; compared as sets below
        assert_bits_equal(got, g[f"{case}/{name}"], name)
    for got, name in zip(rec, ("tree_prefix", "tree_depth", "tree_mass", "tree_com")):
        if case == "duplicate_key" and name in ("tree_mass", "tree_com"):
            continue  # leaf sums depend on the tie order
        assert_bits_equal(got, g[f"{case}/{name}"], name)
    if case != "duplicate_key":
        assert_bits_equal(acc, g[f"{case}/acc"], "acc")


def test_duplicate_key_ties_as_sets(port, golden):
    g = golden("edge_cases.npz")
    c = "duplicate_key"
    pos, vel, mass, ids = (g[f"{c}/{k}"] for k in ("pos", "vel", "mass", "ids"))
    _, _, (sk, sp, sm, sv, si), rec, acc = run_stages(port, pos, vel, mass, ids)
    ref_ids = g[f"{c}/sorted_ids"]
    ref_keys = g[f"{c}/sorted_keys"]
    for k in np.unique(ref_keys):
        assert set(si[sk == k]) == set(ref_ids[ref_keys == k])
    assert len(np.unique(ref_keys)) == len(ref_keys) - 1
    # masses/COMs of the tree agree to rounding whatever the tie order
    np.testing.assert_allclose(rec[2], g[f"{c}/tree_mass"], rtol=1e-15)
    np.testing.assert_allclose(rec[3], g[f"{c}/tree_com"], rtol=1e-13, atol=1e-300)
    np.testing.assert_allclose(acc, g[f"{c}/acc"], rtol=1e-12, atol=1e-30)


def test_synthetic_1000_bit_exact(port, golden):
    g = golden("synthetic_1000.npz")
    pos, vel, mass, ids = g["pos"], g["vel"], g["mass"], g["ids"]
    bb, keys, srt, rec, acc = run_stages(port, pos, vel, mass, ids)
    assert_bits_equal(bb, g["bbox"], "bbox")
    assert_bits_equal(keys, g["keys"], "keys")
    for got, name in zip(srt, ("sorted_keys", "sorted_pos", "sorted_mass", "sorted_vel", "sorted_ids")):
        assert_bits_equal(got, g[name], name)
    for got, name in zip(rec, ("tree_prefix", "tree_depth", "tree_mass", "tree_com")):
        assert_bits_equal(got, g[name], name)
    assert_bits_equal(acc, g["acc"], "acc")
    for th in (0.5, 0.8):
        *_, a = run_stages(port, pos, vel, mass, ids, theta=th)
        assert_bits_equal(a, g[f"acc_theta_{th}"], f"acc theta={th}")


def test_synthetic_1000_five_steps(port, golden):
    g = golden("synthetic_1000.npz")
    p, v, m, i, a, t, _ = port.simulate(g["pos"], g["vel"], g["mass"], g["ids"], DT, THETA, G, 5)
    for got, name in zip((p, v, m, i, a), ("sim5_pos", "sim5_vel", "sim5_mass", "sim5_ids", "sim5_acc")):
        assert_bits_equal(got, g[name], name)
    assert t == g["sim5_t"][0]


def test_synthetic_19054_digests(port, golden):
    g = golden("synthetic_19054.npz")
    pos, vel, mass, ids = g["pos"], g["vel"], g["mass"], g["ids"]
    bb, keys, (sk, sp, sm, sv, si), rec, acc = run_stages(port, pos, vel, mass, ids)
    assert_bits_equal(bb, g["bbox"], "bbox")
    assert_bits_equal(keys, g["keys"], "keys")
    assert_bits_equal(si, g["sorted_ids"], "permutation")
    assert len(rec[0]) == int(g["n_records"][0])
    assert np.array_equal(np.bincount(rec[1], minlength=22), g["depth_hist"])
    assert digest(*rec) == str(g["tree_digest"][0])
    assert digest(acc) == str(g["acc_digest"][0])
    assert_bits_equal(acc[:512], g["acc_head"], "acc head")
    p, v, m, i, a, t, _ = port.simulate(pos, vel, mass, ids, DT, THETA, G, 3)
    assert digest(p, v, m, i, a) == str(g["sim3_digest"][0])
    assert t == g["sim3_t"][0]


def test_step_count_semantics(port, golden):
    """`for (t = 0; t < t_end; t += dt)` with dt = 1h: 10 d -> 241 steps."""
    t, steps = 0.0, 0
    while t < 10.0:
        steps += 1
        t += 1.0 / 24.0
    assert steps == 241


from oracle.oracle import REF_SRC  # noqa: E402  (where the reference checkout lives, if anywhere)

REF_CSV = REF_SRC / "data" / "state_vectors_csvs" / "scenario1_19054.csv"


@pytest.mark.skipif(not REF_CSV.exists(), reason="the reference checkout is not on this host")
def test_scenario1_csv_digests(port, bh):
    info = json.loads((GOLDEN / "scenario1.json").read_text())
    ids, mass, pos, vel = bh.read_csv(REF_CSV)
    assert len(mass) == info["n"]
    assert digest(pos, vel, mass, ids) == info["input_digest"]
    bb, keys, (sk, sp, sm, sv, si), rec, acc = run_stages(port, pos, vel, mass, ids)
    assert bb.tolist() == info["bbox"]
    assert digest(keys) == info["keys_digest"]
    assert digest(si) == info["sorted_ids_digest"]
    assert len(rec[0]) == info["n_records"]
    assert np.bincount(rec[1], minlength=22).tolist() == info["depth_hist"]
    assert digest(*rec) == info["tree_digest"]
    assert digest(acc) == info["acc_digest"]


@pytest.mark.skipif(not (REF_SRC / "src" / "traversal.cpp").exists(), reason="reference checkout absent")
def test_port_equals_compiled_reference_random(port):
    """Random systems, several theta: the port and the compiled reference agree bit for bit."""
    from oracle.oracle import Oracle, build_reference
    build_reference()
    ref = Oracle("reference")
    rng = np.random.default_rng(5)
    for n, theta in ((3, 1.05), (17, 0.3), (300, 0.7), (2500, 1.05), (2500, 2.0)):
        pos = rng.standard_normal((n, 3)) * rng.uniform(0.1, 30, (n, 1))
        vel = rng.standard_normal((n, 3)) * 1e-3
        mass = 10 ** rng.uniform(12, 25, n)
        ids = np.arange(n, dtype=np.uint64)
        a = run_stages(port, pos, vel, mass, ids, theta)
        b = run_stages(ref, pos, vel, mass, ids, theta)
        assert_bits_equal(a[0], b[0], "bbox")
        assert_bits_equal(a[1], b[1], "keys")
        for x, y in zip(a[2], b[2]):
            assert_bits_equal(x, y, "sorted")
        for x, y in zip(a[3], b[3]):
            assert_bits_equal(x, y, "tree")
        assert_bits_equal(a[4], b[4], "acc")
    el = np.column_stack([rng.uniform(0, 0.9, 50), rng.uniform(0.3, 50, 50), rng.uniform(0, 3, 50),
                          rng.uniform(0, 6.3, 50), rng.uniform(0, 6.3, 50), rng.uniform(-7, 7, 50),
                          rng.uniform(2451000, 2452000, 50), np.full(50, 2.96e-4)])
    assert_bits_equal(port.kepler(el), ref.kepler(el), "kepler")


def _let_tree(o, g, local, bb):
    """The local tree of buildOctreeBottomUp (no merge) over the bodies in
    `local`, keys in the global box `bb`."""
    sel = np.nonzero(local)[0]
    keys = o.keys(g["pos"][sel], bb)
    sk, sp, sm, _, _, _ = o.sort(keys, g["pos"][sel], g["mass"][sel], g["vel"][sel], g["ids"][sel])
    return o.tree(sk, sp, sm, merge=False)


@pytest.mark.parametrize("system", ["synthetic_1000", "synthetic_19054"])
def test_let_export_matches_reference(port, golden, system):
    """createInteractionListForRank restated in the oracle against the
    compiled reference's exports (bucket domains of other ranks and random
    boxes; theta 0.3-1.5; max_depth 0, 4, 21, 25)."""
    g = golden(f"{system}.npz")
    f = golden("let_export.npz")
    bb = f[f"{system}/bbox"]
    for ci in range(int(f[f"{system}/n_cases"][0])):
        c = f"{system}/c{ci}/"
        local = np.unpackbits(f[c + "local"])[:len(g["mass"])].astype(bool)
        tree = _let_tree(port, g, local, bb)
        p, d, m, com = port.let_export(tree, f[c + "boxes"], bb, float(f[c + "theta2"][0]), int(f[c + "max_depth"][0]))
        tree.close()
        assert len(p) == int(f[c + "count"][0]), ci
        h = hashlib.sha256()
        for a in (p, d, m, com):
            h.update(np.ascontiguousarray(a).tobytes())
        assert h.hexdigest() == str(f[c + "digest"][0]), ci
        if c + "prefix" in f:
            assert_bits_equal(p, f[c + "prefix"], f"case {ci} prefixes")
            assert_bits_equal(com, f[c + "com"], f"case {ci} centres of mass")


def test_pseudo_tree_matches_reference(port, golden):
    """buildTreeFromPseudoLeaves restated in the oracle (children summed in
    octant order) against the compiled reference (hash-map order): the same
    cells; masses and centres of mass within 1e-14 relative."""
    f = golden("pseudo_tree.npz")
    t = port.pseudo_tree(f["prefix"], f["depth"], f["mass"], f["com"])
    p, d, m, c = t.records()
    t.close()
    assert_bits_equal(p, f["tree_prefix"], "prefixes")
    assert_bits_equal(d, f["tree_depth"], "depths")
    assert np.all(np.abs(m - f["tree_mass"]) <= 1e-14 * np.abs(f["tree_mass"]))
    scale = np.abs(f["tree_com"]).max(axis=1, keepdims=True)
    assert np.all(np.abs(c - f["tree_com"]) <= 1e-14 * scale)
    # cells whose sums involve no reordering agree bit for bit
    assert np.mean(m == f["tree_mass"]) > 0.8


def _rank0_tree(o, f, g):
    local = np.unpackbits(f["local"])[:len(g["mass"])].astype(bool)
    sel = np.nonzero(local)[0]
    bb = f["bbox"]
    keys = o.keys(g["pos"][sel], bb)
    sk, sp, sm, _, _, _ = o.sort(keys, g["pos"][sel], g["mass"][sel], g["vel"][sel], g["ids"][sel])
    return o.tree(sk, sp, sm, merge=False), sk, sp


def test_let_forces_match_reference(port, golden):
    """computeAccelerationsWithLET and ...WithRemoteDirectSum restated in the
    oracle against the compiled reference (rank 0 of a 4-way split of the
    1,000-body system): within 1e-13 relative (the pseudo-leaf map's child
    sums are the only order difference)."""
    f = golden("pseudo_tree.npz")
    g = golden("synthetic_1000.npz")
    nv = int(f["n_valid"][0])
    rec = (f["prefix"], f["depth"], f["mass"], f["com"])
    valid = tuple(a[:nv] for a in rec)
    tree, sk, sp = _rank0_tree(port, f, g)
    got = {"let_acc": port.let_accelerations(tree, valid, sk, sp, THETA, G, f["bbox"]),
           "let_acc_all": port.let_accelerations(tree, rec, sk, sp, THETA, G, f["bbox"]),
           "letds_acc": port.let_accelerations(tree, valid, sk, sp, THETA, G, f["bbox"], direct=True)}
    tree.close()
    for k, a in got.items():
        want = f[k]
        rel = np.linalg.norm(a - want, axis=1) / np.linalg.norm(want, axis=1)
        assert rel.max() <= 1e-13, k


def test_oracle_generator_matches_engine(bh, port):
    """The oracle's restatement of the seeded generator (used by the bench's
    reference arm, which must not load the engine's library) gives the
    engine's bodies bit for bit: every configuration's mix, small sizes and
    odd fractions."""
    from conftest import assert_bits_equal
    for seed, n, outer, trojan in ((2, 300_149, 0.1, 0.0), (5, 100_000, 0.10, 0.05), (1, 19_054, 0.0, 0.0),
                                   (7, 1000, 0.1, 0.05), (3, 9, 0.0, 0.0), (4, 12, 0.5, 0.5)):
        got = port.generate_system(seed, n, outer, trojan)
        want = bh.generate_system(seed, n, outer, trojan)
        for a, b, name in zip(got, want, ("pos", "vel", "mass", "ids")):
            assert_bits_equal(a, b, f"seed {seed} n {n} {name}")
