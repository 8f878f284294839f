"""Generates the golden fixtures in this folder from the reference's own
sources, compiled unmodified by ``make -C oracle ref`` (oracle/_ref).

Run in a checkout where the reference is present:

    python tests/golden/make_golden.py [edge synthetic let pseudo config1 scenario]

(no arguments: every fixture).

Outputs (all produced by the compiled reference, strict IEEE build):

* ``edge_cases.npz``      -- hand-made small systems (N = 1, 2, a duplicate
                             key, a coplanar and a single-point system, a
                             massless body, the 9 massive bodies): inputs and
                             every stage's full output.
* ``synthetic_1000.npz``  -- seeded synthetic system (seed 7, 1,000 bodies,
                             10 % outer belt, 5 % trojans): inputs, every
                             stage's full output (the tree also without the
                             single-rank merge) and 5 steps of the loop.
* ``synthetic_19054.npz`` -- the CPU-runnable workload (seed 1, 19,054 bodies:
                             Sun, 8 planets, 19,045 inner-belt asteroids):
                             inputs, keys, permutation, SHA-256 digests of the
                             tree and of the accelerations, and the first 512
                             accelerations in full.
* ``let_export.npz``      -- createInteractionListForRank on the tree of
                             buildOctreeBottomUp (no merge) of the two
                             synthetic systems above (their inputs are read
                             from those files): remote domains of bucket boxes
                             (key-range splits as update_rank_domains makes
                             them) and of random boxes, several theta and
                             max_depth values; the kept cells sorted by
                             (depth, prefix).
* ``pseudo_tree.npz``     -- buildTreeFromPseudoLeaves over the records rank 0
                             of a 4-way split of synthetic_1000 receives
                             (the other ranks' exports to its bucket boxes),
                             plus duplicate, massless, non-finite, negative,
                             unmasked and too-deep records: inputs and the
                             map, sorted by (depth, prefix); rank 0's forces
                             from computeAccelerationsWithLET (with and without
                             the edge records) and
                             computeAccelerationsWithRemoteDirectSum.
* ``config1_240_steps.json`` -- the CPU-runnable configuration's full run:
                             240 steps of 1 h at theta 1.05 from the inputs of
                             synthetic_19054.npz; SHA-256 of the final state
                             (pos, vel, mass, ids, acc in the final sorted
                             order) and the final time.
* ``scenario1.json``      -- digests of the same stages on the reference's own
                             data/state_vectors_csvs/scenario1_19054.csv, read
                             by the reference's readCSV (the file itself is not
                             copied here).
* ``io.npz``              -- the reference's I/O code (src/io.cpp, compiled by
                             the same recipe): readCSV on the seeded CSV files
                             of csv_cases.py (counts, digests, warnings; full
                             arrays for the small files); the bytes
                             writeSnapshot writes for a state of awkward values;
                             the .pvd updatePVDFile builds over three frames;
                             and the reference driver (main.cpp, one rank, tree
                             path) run on a 1,000-body CSV: every snapshot and
                             .pvd file it writes, final_ref.csv of a -r run and
                             SUMMED_DIST_ERROR of a rerun against it.

Inputs of the synthetic systems come from the engine's generator
(``bh_generate_system``) and are stored, so the fixtures do not depend on the
platform's libm.
"""
from __future__ import annotations

import contextlib
import hashlib
import importlib
import json
import os
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle.oracle import REF_SRC, Oracle, build_reference  # noqa: E402

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
import csv_cases  # noqa: E402

G = 1.48812e-34
THETA = 1.05
DT = 1.0 / 24.0


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def stages(ref: Oracle, pos, vel, mass, ids, theta=THETA):
    """Every stage of one force evaluation, as the reference computes it."""
    bb = ref.bbox(pos)
    keys = ref.keys(pos, bb)
    sk, sp, sm, sv, si, _ = ref.sort(keys, pos, mass, vel, ids)
    tree = ref.tree(sk, sp, sm, merge=True)
    prefix, depth, tmass, com = tree.records()
    acc = ref.accelerations(tree, sk, sp, theta, G, 0.0, bb)
    tree.close()
    return dict(bbox=bb, keys=keys, sorted_keys=sk, sorted_pos=sp, sorted_mass=sm, sorted_vel=sv,
                sorted_ids=si, tree_prefix=prefix, tree_depth=depth, tree_mass=tmass, tree_com=com, acc=acc)


def edge_systems():
    rng = np.random.default_rng(11)
    cases = {}
    cases["one"] = (np.array([[0.5, -0.25, 1.0]]), np.array([[0.01, 0.0, 0.0]]), np.array([3.0e20]))
    cases["two"] = (np.array([[0.0, 0.0, 0.0], [1.0, 0.5, -0.5]]), np.zeros((2, 3)), np.array([1.989e30, 5.97e24]))
    p = rng.uniform(-3, 3, (40, 3)); p[17] = p[5]  # two bodies share a position -> duplicate key
    cases["duplicate_key"] = (p, rng.normal(0, 0.01, (40, 3)), rng.uniform(1e15, 1e20, 40))
    p = rng.uniform(-3, 3, (64, 3)); p[:, 2] = 0.0  # degenerate z span
    cases["coplanar"] = (p, rng.normal(0, 0.01, (64, 3)), rng.uniform(1e15, 1e20, 64))
    p = np.tile([[1.5, -2.0, 0.25]], (5, 1))  # every body at one point
    cases["single_point"] = (p, np.zeros((5, 3)), np.full(5, 1e18))
    p = rng.uniform(-3, 3, (50, 3)); m = rng.uniform(1e15, 1e20, 50); m[3] = 0.0; m[30] = 0.0
    cases["massless"] = (p, rng.normal(0, 0.01, (50, 3)), m)
    return cases


def bucket_boxes(prefixes, bucket_bits, bb):
    """exchangeEssentialTrees' bucket boxes (src/exchange.cpp:45-71) in the
    same float64 operation order (numpy rounds each operation, no FMA)."""
    d = bucket_bits // 3
    bits = np.asarray(prefixes, np.uint64) >> np.uint64(63 - 3 * d) if d else np.zeros(len(prefixes), np.uint64)
    out = np.empty((len(prefixes), 6))
    scale = 1.0 / float(1 << d)
    for a in range(3):
        v = np.zeros(len(prefixes), np.uint64)
        for b in range(d):
            v |= ((bits >> np.uint64(3 * b + a)) & np.uint64(1)) << np.uint64(b)
        span = bb[3 + a] - bb[a]
        lo = bb[a] + (v.astype(np.float64) * scale) * span
        out[:, a] = lo
        out[:, 3 + a] = lo + span / float(1 << d)
    return out


def let_cases(ref: Oracle, pos, vel, mass, ids, rng, full: bool):
    """LET exports of one system for a few remote domains.  Bucket cases:
    the bodies are split into contiguous bucket ranges of about n / nranks
    bodies (as update_rank_domains, src/load_balancing.cpp:12-65, splits
    them); rank 0's bodies form the local tree (keys in the global box) and
    each other rank's non-empty buckets its domain.  Random cases: all bodies
    are local, the domain is a few random boxes.  With `full` the kept cells
    are stored, otherwise their count, depth histogram and SHA-256 digest."""
    n = len(mass)
    bb = ref.bbox(pos)
    keys = ref.keys(pos, bb)
    out = {"bbox": bb}
    cases = []
    for bucket_bits, nranks in ((6, 2), (9, 4), (12, 3)):
        bidx = (keys >> np.uint64(63 - bucket_bits)).astype(np.int64)
        hist = np.bincount(bidx, minlength=1 << bucket_bits)
        ideal = (n + nranks - 1) // nranks
        split, run = [], 0
        for i, h in enumerate(hist):
            run += int(h)
            if len(split) < nranks - 1 and run >= (len(split) + 1) * ideal:
                split.append(i)
        owner = np.searchsorted(np.array(split, np.int64), np.arange(1 << bucket_bits), side="right")
        local = owner[bidx] == 0
        for r in range(1, nranks):
            pref = (np.nonzero((hist > 0) & (owner == r))[0].astype(np.uint64)) << np.uint64(63 - bucket_bits)
            cases.append((bucket_boxes(pref, bucket_bits, bb), local, pref, bucket_bits))
    for _ in range(4):
        k = int(rng.integers(1, 6))
        c = rng.uniform(bb[:3], bb[3:], (k, 3)); h = rng.uniform(0.2, 15.0, (k, 3))
        cases.append((np.concatenate([c - h, c + h], axis=1), np.ones(n, bool), None, -1))
    params = ((1.05, 21), (0.5, 21), (1.05, 4), (0.3, 0), (1.5, 25), (0.7, 21))
    for ci, (boxes, local, pref, bits) in enumerate(cases):
        theta, max_depth = params[ci % len(params)]
        sel = np.nonzero(local)[0]
        sk, sp, sm, _, _, _ = ref.sort(keys[sel], pos[sel], mass[sel], vel[sel], ids[sel])
        tree = ref.tree(sk, sp, sm, merge=False)
        p, d, m, c = ref.let_export(tree, boxes, bb, theta * theta, max_depth)
        tree.close()
        out[f"c{ci}/local"] = np.packbits(local)
        out[f"c{ci}/boxes"] = boxes
        out[f"c{ci}/theta2"] = np.array([theta * theta])
        out[f"c{ci}/max_depth"] = np.array([max_depth])
        if pref is not None:
            out[f"c{ci}/bucket_prefixes"] = pref
            out[f"c{ci}/bucket_bits"] = np.array([bits])
        out[f"c{ci}/count"] = np.array([len(p)])
        out[f"c{ci}/depth_hist"] = np.bincount(d, minlength=22)
        out[f"c{ci}/digest"] = np.array([digest(p, d, m, c)])
        if full:
            out[f"c{ci}/prefix"] = p; out[f"c{ci}/depth"] = d; out[f"c{ci}/mass"] = m; out[f"c{ci}/com"] = c
    out["n_cases"] = np.array([len(cases)])
    return out


def main() -> None:
    if build_reference() is None:
        raise SystemExit("the reference checkout is needed to regenerate the fixtures")
    ref = Oracle("reference")
    bh = importlib.import_module("barnes-hut_gb300")
    want = set(sys.argv[1:]) or {"edge", "synthetic", "let", "pseudo", "config1", "scenario", "io"}
    if "edge" in want:
        edge_fixtures(ref, bh)
    if "synthetic" in want:
        synthetic_fixtures(ref, bh)
    if "let" in want:
        let_fixtures(ref, bh)
    if "pseudo" in want:
        pseudo_fixtures(ref)
    if "config1" in want:
        config1_fixture(ref)
    if "scenario" in want:
        scenario_fixture(ref)
    if "io" in want:
        io_fixtures(ref)
    print("fixtures written to", HERE)


def edge_fixtures(ref, bh):
    out = {}
    for name, (pos, vel, mass) in edge_systems().items():
        ids = np.arange(len(mass), dtype=np.uint64)
        out[f"{name}/pos"] = pos; out[f"{name}/vel"] = vel; out[f"{name}/mass"] = mass; out[f"{name}/ids"] = ids
        for k, v in stages(ref, pos, vel, mass, ids).items():
            out[f"{name}/{k}"] = v
    pos, vel, mass, ids = bh.generate_system(3, 9, 0.0, 0.0)
    out["massive/pos"] = pos; out["massive/vel"] = vel; out["massive/mass"] = mass; out["massive/ids"] = ids
    for k, v in stages(ref, pos, vel, mass, ids).items():
        out[f"massive/{k}"] = v
    np.savez_compressed(HERE / "edge_cases.npz", **out)


def synthetic_fixtures(ref, bh):
    # Synthetic 1,000
    pos, vel, mass, ids = bh.generate_system(7, 1000, 0.1, 0.05)
    out = dict(pos=pos, vel=vel, mass=mass, ids=ids)
    out.update(stages(ref, pos, vel, mass, ids))
    for th in (0.5, 0.8):
        out[f"acc_theta_{th}"] = stages(ref, pos, vel, mass, ids, theta=th)["acc"]
    # buildOctreeBottomUp alone (no single-rank exchange merge)
    t_nm = ref.tree(out["sorted_keys"], out["sorted_pos"], out["sorted_mass"], merge=False)
    for k, v in zip(("prefix", "depth", "mass", "com"), t_nm.records()):
        out[f"tree_nomerge_{k}"] = v
    t_nm.close()
    p, v, m, i, a, t, _ = ref.simulate(pos, vel, mass, ids, DT, THETA, G, 5)
    out.update(sim5_pos=p, sim5_vel=v, sim5_mass=m, sim5_ids=i, sim5_acc=a, sim5_t=np.array([t]))
    np.savez_compressed(HERE / "synthetic_1000.npz", **out)

    # Synthetic 19,054 (the CPU-runnable workload)
    pos, vel, mass, ids = bh.generate_system(1, 19054, 0.0, 0.0)
    s = stages(ref, pos, vel, mass, ids)
    sk, sp, sm, sv, si, _ = ref.sort(s["keys"], pos, mass, vel, ids)
    out = dict(pos=pos, vel=vel, mass=mass, ids=ids, bbox=s["bbox"], keys=s["keys"], sorted_ids=si,
               n_records=np.array([len(s["tree_mass"])]),
               depth_hist=np.bincount(s["tree_depth"], minlength=22),
               tree_digest=np.array([digest(s["tree_prefix"], s["tree_depth"], s["tree_mass"], s["tree_com"])]),
               acc_digest=np.array([digest(s["acc"])]), acc_head=s["acc"][:512])
    p, v, m, i, a, t, _ = ref.simulate(pos, vel, mass, ids, DT, THETA, G, 3)
    out.update(sim3_digest=np.array([digest(p, v, m, i, a)]), sim3_t=np.array([t]))
    np.savez_compressed(HERE / "synthetic_19054.npz", **out)


def let_fixtures(ref, bh):
    # Locally essential tree exports
    rng = np.random.default_rng(2024)
    out = {}
    for tag in ("synthetic_1000", "synthetic_19054"):
        g = np.load(HERE / f"{tag}.npz")
        for k, v in let_cases(ref, g["pos"], g["vel"], g["mass"], g["ids"], rng, tag == "synthetic_1000").items():
            out[f"{tag}/{k}"] = v
    np.savez_compressed(HERE / "let_export.npz", **out)


def pseudo_fixtures(ref):
    g = np.load(HERE / "synthetic_1000.npz")
    pos, vel, mass, ids = g["pos"], g["vel"], g["mass"], g["ids"]
    bb = ref.bbox(pos)
    keys = ref.keys(pos, bb)
    bits, nranks = 6, 4
    bidx = (keys >> np.uint64(63 - bits)).astype(np.int64)
    hist = np.bincount(bidx, minlength=1 << bits)
    ideal = (len(keys) + nranks - 1) // nranks
    split, run = [], 0
    for i, h in enumerate(hist):
        run += int(h)
        if len(split) < nranks - 1 and run >= (len(split) + 1) * ideal:
            split.append(i)
    owner = np.searchsorted(np.array(split, np.int64), np.arange(1 << bits), side="right")
    pref0 = (np.nonzero((hist > 0) & (owner == 0))[0].astype(np.uint64)) << np.uint64(63 - bits)
    boxes0 = bucket_boxes(pref0, bits, bb)
    parts = []
    for r in range(1, nranks):
        sel = np.nonzero(owner[bidx] == r)[0]
        sk, sp, sm, _, _, _ = ref.sort(keys[sel], pos[sel], mass[sel], vel[sel], ids[sel])
        tree = ref.tree(sk, sp, sm, merge=False)
        parts.append(ref.let_export(tree, boxes0, bb, 0.5 ** 2, 21))
        tree.close()
    p = np.concatenate([x[0] for x in parts]); d = np.concatenate([x[1] for x in parts])
    m = np.concatenate([x[2] for x in parts]); c = np.concatenate([x[3] for x in parts])
    n_valid = len(p)
    # rank 0's forces with these records: computeAccelerationsWithLET and
    # computeAccelerationsWithRemoteDirectSum over its local tree (bodies in
    # sorted key order)
    local = owner[bidx] == 0
    sel = np.nonzero(local)[0]
    sk, sp, sm, _, _, _ = ref.sort(keys[sel], pos[sel], mass[sel], vel[sel], ids[sel])
    tree = ref.tree(sk, sp, sm, merge=False)
    let_acc = ref.let_accelerations(tree, (p, d, m, c), sk, sp, THETA, G, bb)
    letds_acc = ref.let_accelerations(tree, (p, d, m, c), sk, sp, THETA, G, bb, direct=True)
    tree.close()
    # edge records: a duplicate key (summed in input order), massless,
    # non-finite and negative masses (skipped), an unmasked prefix, depth 30
    p = np.concatenate([p, p[:3], p[3:6], [p[6] | np.uint64(0x5555)], [p[7]]])
    d = np.concatenate([d, d[:3], d[3:6], [d[6]], [30]]).astype(np.uint8)
    m = np.concatenate([m, m[:3] * 0.25, [0.0, np.nan, -m[5]], [m[6]], [m[7]]])
    c = np.concatenate([c, c[:3] * 0.5, c[3:6], c[6:7], c[7:8]])
    out = dict(prefix=p, depth=d, mass=m, com=c, n_valid=np.array([n_valid]), local=np.packbits(local), bbox=bb)
    # the forces again with the edge records (the pseudo-leaf map skips them)
    sk, sp, sm, _, _, _ = ref.sort(keys[sel], pos[sel], mass[sel], vel[sel], ids[sel])
    tree = ref.tree(sk, sp, sm, merge=False)
    out["let_acc_all"] = ref.let_accelerations(tree, (p, d, m, c), sk, sp, THETA, G, bb)
    tree.close()
    out["let_acc"] = let_acc
    out["letds_acc"] = letds_acc
    t = ref.pseudo_tree(p, d, m, c)
    for k, v in zip(("prefix", "depth", "mass", "com"), t.records()):
        out[f"tree_{k}"] = v
    t.close()
    np.savez_compressed(HERE / "pseudo_tree.npz", **out)


def config1_fixture(ref):
    g = np.load(HERE / "synthetic_19054.npz")
    p, v, m, i, a, t, _ = ref.simulate(g["pos"], g["vel"], g["mass"], g["ids"], DT, THETA, G, 240)
    info = dict(steps=240, dt=DT, theta=THETA, G=G, t=t, digest=digest(p, v, m, i, a),
                pos_head=p[:4].tolist())
    (HERE / "config1_240_steps.json").write_text(json.dumps(info, indent=1) + "\n")


def scenario_fixture(ref):
    # The reference's own scenario-1 CSV, read by its readCSV: digests only.
    csv = REF_SRC / "data" / "state_vectors_csvs" / "scenario1_19054.csv"
    if csv.exists():
        ids, mass, pos, vel = ref.read_csv(csv)
        s = stages(ref, pos, vel, mass, ids)
        info = dict(n=int(len(mass)), input_digest=digest(pos, vel, mass, ids), bbox=s["bbox"].tolist(),
                    keys_digest=digest(s["keys"]), sorted_ids_digest=digest(s["sorted_ids"]),
                    n_records=int(len(s["tree_mass"])),
                    depth_hist=np.bincount(s["tree_depth"], minlength=22).tolist(),
                    duplicate_keys=int(len(s["keys"]) - len(np.unique(s["keys"]))),
                    tree_digest=digest(s["tree_prefix"], s["tree_depth"], s["tree_mass"], s["tree_com"]),
                    acc_digest=digest(s["acc"]))
        (HERE / "scenario1.json").write_text(json.dumps(info, indent=1) + "\n")


@contextlib.contextmanager
def captured_stderr(lines: list):
    """Collects what C++ code writes to fd 2 (std::cerr) into `lines`."""
    sys.stderr.flush()
    saved = os.dup(2)
    with tempfile.TemporaryFile() as tmp:
        os.dup2(tmp.fileno(), 2)
        try:
            yield
        finally:
            os.dup2(saved, 2)
            os.close(saved)
            tmp.seek(0)
            lines.extend(tmp.read().decode(errors="replace").splitlines())


def awkward_state(n=50, seed=3):
    """A state with values the number formatting must get right: wide
    exponents, signed zeros, inf/nan, a subnormal, large ids."""
    rng = np.random.default_rng(seed)
    pos = rng.normal(0, 3, (n, 3)) * 10.0 ** rng.integers(-12, 12, (n, 3))
    vel = rng.normal(0, 1e-2, (n, 3))
    acc = rng.normal(0, 1e-5, (n, 3))
    pos[0] = [-0.0, 0.0, 1e300]
    vel[1] = [np.inf, -np.inf, np.nan]
    acc[2] = [1e-310, 0.0, 0.0]
    acc[3] = [1e200, 1e200, 0.0]  # |a| overflows to inf
    mass = rng.uniform(1e15, 1e25, n)
    mass[4] = 0.0
    ids = np.arange(n, dtype=np.uint64) * np.uint64(1 << 40) + np.uint64(7)
    return ids, mass, pos, vel, acc


# The reference driver runs the I/O fixtures pin: (name, command line).  The
# input is bodies.csv (synthetic_1000's state); runs share one directory, so
# the rerun finds the -r run's reference/final_ref.csv.
CLI_RUNS = (
    ("frames", ["-f", "bodies.csv", "--dt", "1h", "--tend", "1d", "--vs", "6h", "-o", "frames", "--fc", "tree"]),
    ("limit", ["-f", "bodies.csv", "--dt", "2h", "--tend", "12h", "--vs", "4h", "-o", "limit", "-b", "400",
               "--theta", "0.8", "--fc", "tree"]),
    ("reference", ["-f", "bodies.csv", "--dt", "1h", "--tend", "6h", "--vs", "1d", "-o", "ref_out", "--fc", "tree",
                   "-r"]),
    ("rerun", ["-f", "bodies.csv", "--dt", "1h", "--tend", "6h", "--vs", "1d", "-o", "rerun_out", "--theta", "0.5",
               "--fc", "tree"]),
)


def io_fixtures(ref):
    out = {}
    with tempfile.TemporaryDirectory() as d:
        d = Path(d)
        # readCSV (src/io.cpp:16-81)
        for name, (make_rows, crlf, final_nl, limits) in csv_cases.cases().items():
            f = d / f"{name}.csv"
            out[f"csv/{name}/sha256"] = np.array([csv_cases.write(f, make_rows(), crlf, final_nl)])
            for lim in limits:
                warn = []
                with captured_stderr(warn):
                    ids, mass, pos, vel = ref.read_csv(f, lim)
                key = f"csv/{name}/lim{lim}"
                out[f"{key}/n"] = np.array([len(mass)])
                out[f"{key}/digest"] = np.array([digest(ids, mass, pos, vel)])
                out[f"{key}/warnings"] = np.array(["\n".join(warn)])
                if len(mass) <= 4000:
                    out[f"{key}/ids"] = ids; out[f"{key}/mass"] = mass; out[f"{key}/pos"] = pos
                    out[f"{key}/vel"] = vel
        for name, data in (("empty", b""), ("header_only", csv_cases.HEADER.encode()),
                           ("header_newline", (csv_cases.HEADER + "\n").encode())):
            f = d / f"{name}.csv"
            f.write_bytes(data)
            out[f"csv/{name}/n"] = np.array([len(ref.read_csv(f)[1])])
        # writeSnapshot (src/io.cpp:84-232): rank 3, counter 2; and an empty state
        ids, mass, pos, vel, acc = awkward_state()
        ref.write_snapshot(3, 2, ids, mass, pos, vel, acc, d / "snap")
        out.update({"vtp/ids": ids, "vtp/mass": mass, "vtp/pos": pos, "vtp/vel": vel, "vtp/acc": acc,
                    "vtp/bytes": np.frombuffer((d / "snap" / "3" / "sim.2.vtp").read_bytes(), np.uint8)})
        ref.write_snapshot(0, 0, ids[:0], mass[:0], pos[:0], vel[:0], acc[:0], d / "empty")
        out["vtp/empty_writes_file"] = np.array([(d / "empty" / "0" / "sim.0.vtp").exists()])
        # updatePVDFile (src/io.cpp:234-298) over three frames
        args = ["-f", "data/bodies.csv", "--dt", "1h", "--tend", "10d", "--theta", "0.8", "-b", "500", "--fc", "tree"]
        times = (0.0, 0.29166666666666663, 10.0 / 3.0)
        (d / "pvd").mkdir()  # the driver creates it (main.cpp:125)
        for k, t in enumerate(times):
            ref.update_pvd(args, 1, k, t, d / "pvd")
        (pvd,) = (d / "pvd").glob("*.pvd")
        out.update({"pvd/args": np.array(args), "pvd/times": np.array(times), "pvd/name": np.array([pvd.name]),
                    "pvd/bytes": np.frombuffer(pvd.read_bytes(), np.uint8)})
        # The reference driver on one rank (main.cpp, --fc tree)
        g = np.load(HERE / "synthetic_1000.npz")
        run = d / "cli"
        run.mkdir()
        out["cli/bodies_sha256"] = np.array([csv_cases.write_bodies(run / "bodies.csv", g["ids"], g["mass"], g["pos"],
                                                              g["vel"])])
        cwd = os.getcwd()
        os.chdir(run)
        try:
            for name, cli in CLI_RUNS:
                summed, n, steps, frames = ref.run_cli(cli)
                odir = run / cli[cli.index("-o") + 1]
                files = sorted(str(p.relative_to(odir)) for p in odir.rglob("*") if p.is_file())
                out[f"cli/{name}/args"] = np.array(cli)
                out[f"cli/{name}/summed"] = np.array([summed])
                out[f"cli/{name}/counts"] = np.array([n, steps, frames])
                out[f"cli/{name}/files"] = np.array(files)
                out[f"cli/{name}/sha256"] = np.array([hashlib.sha256((odir / f).read_bytes()).hexdigest()
                                                      for f in files])
                if name == "frames":
                    for f in files:
                        if f.endswith(".pvd") or f == "0/sim.0.vtp":
                            out[f"cli/{name}/bytes/{f}"] = np.frombuffer((odir / f).read_bytes(), np.uint8)
                if name == "reference":
                    out["cli/final_ref_csv"] = np.frombuffer((run / "reference" / "final_ref.csv").read_bytes(),
                                                             np.uint8)
        finally:
            os.chdir(cwd)
        # loadReferenceCSV + computeDistanceSum on their own: the -r file
        # against the 1,000-body state with ids in reverse order
        n = len(g["mass"])
        rp = ref.load_reference_csv(run / "reference", n)
        out["cli/final_ref_loaded"] = rp
        order = np.arange(n)[::-1]
        out["cli/distance_sum_reversed"] = np.array([ref.distance_sum(g["pos"][order], g["ids"][order], rp)])
    np.savez_compressed(HERE / "io.npz", **out)


if __name__ == "__main__":
    main()
