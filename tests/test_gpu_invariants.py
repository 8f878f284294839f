"""Energy and momentum diagnostics: the exact FP64 form against the oracle,
the large-N form (massive-body pairs exact, the rest through the tree) against
the exact form, and the drift of E and L over runs of the step loop in the
FP64 and FP32 forms."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import DT, G, THETA

pytestmark = pytest.mark.gpu


def _ctx(bh, seed, n, outer=0.1, trojan=0.05):
    pos, vel, mass, ids = bh.generate_system(seed, n, outer, trojan)
    c = bh.Context(n)
    c.set_bodies(pos, vel, mass, ids)
    return c, (pos, vel, mass, ids)


def test_exact_matches_oracle(bh, port):
    c, (pos, vel, mass, ids) = _ctx(bh, 21, 5000)
    with c:
        got = c.invariants(G, theta=0.0)
    ref = port.invariants(pos, vel, mass, G)
    # Different summation orders (block partials vs a serial loop): 1e-12.
    for k, key in ((0, "E"), (1, "K"), (2, "U")):
        assert abs(got[key] - ref[k]) <= 1e-12 * abs(ref[k]), key
    scale_l = np.sum(mass * np.linalg.norm(np.cross(pos, vel), axis=1))
    scale_p = np.sum(mass * np.linalg.norm(vel, axis=1))
    assert np.all(np.abs(got["L"] - ref[3:6]) <= 1e-12 * scale_l)
    assert np.all(np.abs(got["P"] - ref[6:9]) <= 1e-12 * scale_p)


def test_tree_form_matches_exact(bh):
    c, _ = _ctx(bh, 22, 100_000)
    with c:
        ex = c.invariants(G, theta=0.0)
        for theta in (0.5, THETA):
            tr = c.invariants(G, theta=theta)
            # Only the asteroid-asteroid part (about 1e-8 of U here) goes
            # through the tree; its theta error is far below 1e-10 of U.
            assert abs(tr["U"] - ex["U"]) <= 1e-10 * abs(ex["U"]), theta
            # K, L, P: the same sums, in the tree's body order after the
            # first tree-form call sorted the bodies (1e-13 relative).
            assert abs(tr["K"] - ex["K"]) <= 1e-13 * ex["K"]
            assert np.linalg.norm(tr["L"] - ex["L"]) <= 1e-13 * np.linalg.norm(ex["L"])
            assert np.linalg.norm(tr["P"] - ex["P"]) <= 1e-13 * np.linalg.norm(ex["P"])


def test_tree_form_at_large_n(bh):
    c, _ = _ctx(bh, 23, 300_000)
    with c:
        with pytest.raises(bh.BhError):
            c.invariants(G, theta=0.0)  # the exact form stops at 131,072 bodies
        inv = c.invariants(G, theta=THETA)
        assert np.isfinite(inv["E"]) and inv["U"] < 0 < inv["K"]
        # the state is still usable: a step after the diagnostic
        c.step(DT, THETA, G, nsteps=1)


def test_drift_over_run(bh):
    """48 steps of 1 h from t = 0, 200,000 bodies with trojans, in the
    reference's FP64 method and in the FP32 far-field form.

    The step loop starts as the reference's does (main.cpp:191-200: no half
    kick at t = 0), which shifts E by about 1.6e-8 of |E| on this system
    (the same shift as a direct-sum leapfrog with that start).  The
    reference's method keeps the Sun and planets in the tree, and monopoles
    of cells that hold a planet break the symmetry of the forces: its CPU
    path moves L by 1.04e-7 of |L| over these 48 steps (measured with the
    oracle on the same system), and the GPU form reproduces it.  The FP32
    form sums the Sun and planets as exact FP64 pair terms, so L stays
    within 1e-9 of its start (measured 1.4e-11) and E within 1e-7."""
    got = {}
    for mode in ("MODE_PLAIN_FP64", "MODE_FP32_FAR"):
        c, _ = _ctx(bh, 24, 200_000)
        with c:
            a = c.invariants(G, theta=THETA)
            c.step(DT, THETA, G, nsteps=48, mode=getattr(bh, mode))
            b = c.invariants(G, theta=THETA)
        de = (b["E"] - a["E"]) / abs(a["E"])
        dl = np.linalg.norm(b["L"] - a["L"]) / np.linalg.norm(a["L"])
        got[mode] = (de, dl)
        print(f"{mode}: dE/|E| = {de:.3g}, |dL|/|L| = {dl:.3g}")
    de, dl = got["MODE_PLAIN_FP64"]
    assert abs(de) < 1e-6 and 5e-8 < dl < 2e-7
    de, dl = got["MODE_FP32_FAR"]
    assert abs(de) < 1e-7 and dl < 1e-9
