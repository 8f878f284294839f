"""Generates the golden fixtures in this folder from the reference's own
sources, compiled unmodified by ``make -C oracle ref`` (oracle/_ref).

Run in a checkout where the reference is present:

    python tests/golden/make_golden.py

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
* ``scenario1.json``      -- digests of the same stages on the reference's own
                             data/state_vectors_csvs/scenario1_19054.csv (the
                             file itself is not copied here).

Inputs of the synthetic systems come from the engine's generator
(``bh_generate_system``) and are stored, so the fixtures do not depend on the
platform's libm.
"""
from __future__ import annotations

import hashlib
import importlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle.oracle import Oracle, build_reference  # noqa: E402

HERE = Path(__file__).resolve().parent
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


def main() -> None:
    if build_reference() is None:
        raise SystemExit("the reference checkout is needed to regenerate the fixtures")
    ref = Oracle("reference")
    bh = importlib.import_module("barnes-hut_gb300")

    # Edge cases
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

    # The reference's own scenario-1 CSV: digests only.
    csv = Path("/root/reference/data/state_vectors_csvs/scenario1_19054.csv")
    if csv.exists():
        ids, mass, pos, vel = bh.read_csv(csv)
        s = stages(ref, pos, vel, mass, ids)
        info = dict(n=int(len(mass)), input_digest=digest(pos, vel, mass, ids), bbox=s["bbox"].tolist(),
                    keys_digest=digest(s["keys"]), sorted_ids_digest=digest(s["sorted_ids"]),
                    n_records=int(len(s["tree_mass"])),
                    depth_hist=np.bincount(s["tree_depth"], minlength=22).tolist(),
                    duplicate_keys=int(len(s["keys"]) - len(np.unique(s["keys"]))),
                    tree_digest=digest(s["tree_prefix"], s["tree_depth"], s["tree_mass"], s["tree_com"]),
                    acc_digest=digest(s["acc"]))
        (HERE / "scenario1.json").write_text(json.dumps(info, indent=1) + "\n")
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
