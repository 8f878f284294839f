"""CPU-side checks of the C ABI library: it loads, exports every function
include/bh_gpu.h declares, and its host-only entry points (Kepler conversion,
synthetic generator, CSV reader/writer) behave like the reference's."""
from __future__ import annotations

import ctypes as C
import re

import numpy as np
import pytest

from conftest import ROOT, assert_bits_equal


def declared_functions():
    text = (ROOT / "include" / "bh_gpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(bh_[a-z_0-9]+)\s*\(", text, flags=re.M)))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("bh_context_create", "bh_compute_keys", "bh_sort_bodies", "bh_build_tree",
                 "bh_compute_accelerations", "bh_step", "bh_export_tree", "bh_generate_morton_codes"):
        assert must in names


def test_library_exports_every_declared_symbol(bh):
    lib = bh.library()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"declared in bh_gpu.h but not exported: {missing}"
    assert lib.bh_api_version() == 1


def test_status_strings(bh):
    lib = bh.library()
    assert lib.bh_status_string(0) == b"ok"
    assert lib.bh_status_string(7) == b"non-finite position"


def test_context_without_gpu_reports_no_device(bh):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(bh.BhError) as e:
        bh.Context(16)
    assert e.value.status == 10  # BH_ERR_NO_DEVICE


def test_invalid_arguments_rejected_without_device(bh):
    lib = bh.library()
    h = C.c_void_p()
    assert lib.bh_context_create(0, 0, C.byref(h)) == 1
    assert lib.bh_context_create(1 << 31, 0, C.byref(h)) == 1
    assert b"capacity" in lib.bh_last_error()
    assert lib.bh_compute_local_bbox(None, -1, None) == 1


def test_kepler_matches_oracle(bh, port):
    rng = np.random.default_rng(3)
    n = 200
    el = np.column_stack([rng.uniform(0, 0.95, n), rng.uniform(0.3, 60, n), rng.uniform(0, 3.1, n),
                          rng.uniform(0, 6.3, n), rng.uniform(0, 6.3, n), rng.uniform(-10, 10, n),
                          rng.uniform(2450000, 2453000, n), np.full(n, 2.95987e-4)])
    assert_bits_equal(bh.kepler_to_cartesian(el), port.kepler(el), "kepler states")


def test_generator_deterministic_and_shaped(bh):
    a = bh.generate_system(42, 5000, 0.1, 0.05)
    b = bh.generate_system(42, 5000, 0.1, 0.05)
    for x, y in zip(a, b):
        assert_bits_equal(x, y)
    pos, vel, mass, ids = a
    assert mass[0] == 1.989e30 and np.all(pos[0] == 0) and np.all(vel[0] == 0)
    r = np.linalg.norm(pos, axis=1)
    np.testing.assert_allclose(r[1:9], [0.3870982252718477, 0.723326849675607, 1.000371833994387,
                                        1.52367818431121, 5.205108585205607, 9.581451990534042,
                                        19.22994588008584, 30.10071183142183], rtol=1e-12)
    assert np.all(pos[1:9, 2] == 0)  # coplanar planets
    nast = 5000 - 9
    n_out, n_tro = round(0.1 * nast), round(0.05 * nast)
    n_in = nast - n_out - n_tro
    inner = r[9:9 + n_in]
    assert inner.min() > 2.1 * (1 - 0.3) - 1e-9 and inner.max() < 3.3 * 1.3 + 1e-9
    outer = r[9 + n_in:9 + n_in + n_out]
    assert outer.min() > 30 * 0.8 - 1e-9 and outer.max() < 50 * 1.2 + 1e-9
    tro = r[9 + n_in + n_out:]
    assert tro.min() > 5.2 * 0.9 - 1e-9 and tro.max() < 5.2 * 1.1 + 1e-9
    # trojans lead/trail Jupiter by 60 +/- 30 degrees in mean longitude; the
    # true position angle differs by up to ~2e rad (e <= 0.1) plus projection
    lam_j = np.arctan2(pos[5, 1], pos[5, 0])
    dl = np.degrees(np.angle(np.exp(1j * (np.arctan2(pos[-n_tro:, 1], pos[-n_tro:, 0]) - lam_j))))
    assert np.all((np.abs(dl) > 15) & (np.abs(dl) < 105))
    m = mass[9:]
    assert m.min() >= 1e12 * (1 - 1e-12) and m.max() <= 1e20 * (1 + 1e-12)
    assert np.array_equal(ids, np.arange(5000, dtype=np.uint64))


def test_csv_round_trip_and_reader_rules(bh, tmp_path):
    pos, vel, mass, ids = bh.generate_system(9, 50, 0.1, 0.0)
    f = tmp_path / "s.csv"
    bh.write_csv(f, ids, mass, pos, vel)
    rid, rmass, rpos, rvel = bh.read_csv(f)
    assert_bits_equal(rpos, pos); assert_bits_equal(rvel, vel); assert_bits_equal(rmass, mass)
    assert np.array_equal(rid, ids)
    # body_count limit, unparsable rows skipped, ids = parsed-row counter
    lines = f.read_text().splitlines()
    bad = lines[:3] + ["7,x,AST,notanumber,1,2,3,4,5,6"] + lines[3:6]
    f.write_text("\n".join(bad) + "\n")
    rid, rmass, rpos, rvel = bh.read_csv(f)
    assert len(rmass) == 5 and np.array_equal(rid, np.arange(5, dtype=np.uint64))
    assert_bits_equal(rmass, np.concatenate([mass[:2], mass[2:5]]))
    rid, rmass, _, _ = bh.read_csv(f, body_count=3)
    assert len(rmass) == 3
    # a row that ends early re-parses its last column (std::getline keeps it)
    f.write_text("h\n0,a,b,5.0,1,2,3,4,5\n")
    _, rmass, rpos, rvel = bh.read_csv(f)
    assert rmass[0] == 5.0 and rvel[0].tolist() == [4.0, 5.0, 5.0]
    with pytest.raises(bh.BhError):
        bh.read_csv(tmp_path / "missing.csv")


def test_vtp_snapshot_layout(bh, tmp_path):
    """bh_write_vtp follows writeSnapshot (io.cpp:84-232): PolyData with the
    position points, rank/body_id/velocity/mass/acceleration-magnitude point
    arrays and one vertex per body, numbers in the default stream format."""
    import xml.etree.ElementTree as ET
    rng = np.random.default_rng(5)
    n = 7
    pos = rng.normal(0, 3, (n, 3)); vel = rng.normal(0, 1e-2, (n, 3)); acc = rng.normal(0, 1e-5, (n, 3))
    mass = rng.uniform(1e15, 1e25, n); ids = np.arange(100, 100 + n, dtype=np.uint64)
    path = tmp_path / "sim.0.vtp"
    bh.write_vtp(path, ids, mass, pos, vel, acc)
    root = ET.parse(path).getroot()
    assert root.tag == "VTKFile" and root.get("type") == "PolyData" and root.get("version") == "0.1"
    piece = root.find("PolyData/Piece")
    assert piece.get("NumberOfPoints") == str(n) and piece.get("NumberOfVerts") == str(n)

    def arr(where, name):
        for da in piece.find(where).findall("DataArray"):
            if da.get("Name") == name:
                return da
        raise AssertionError(name)
    g = lambda v: "%g" % v  # noqa: E731  (the default ostream format: 6 significant digits)
    p = arr("Points", "position")
    assert p.get("type") == "Float64" and p.get("NumberOfComponents") == "3"
    assert p.text.split() == [g(v) for v in pos.ravel()]
    assert arr("PointData", "rank").text.split() == ["0"] * n
    assert arr("PointData", "body_id").text.split() == [str(i) for i in ids]
    assert arr("PointData", "velocity").text.split() == [g(v) for v in vel.ravel()]
    assert arr("PointData", "mass").text.split() == [g(v) for v in mass]
    assert arr("PointData", "acceleration").text.split() == [g(v) for v in np.sqrt((acc ** 2).sum(axis=1))]
    assert arr("Verts", "offsets").text.split() == [str(i) for i in range(1, n + 1)]
    assert arr("Verts", "connectivity").text.split() == [str(i) for i in range(n)]


def test_let_bucket_boxes_match_fixture(bh, golden):
    """bh_let_bucket_boxes reproduces the bucket boxes of the LET fixtures
    (exchangeEssentialTrees' arithmetic) bit for bit."""
    from conftest import assert_bits_equal
    f = golden("let_export.npz")
    seen = 0
    for system in ("synthetic_1000", "synthetic_19054"):
        for ci in range(int(f[f"{system}/n_cases"][0])):
            key = f"{system}/c{ci}/bucket_prefixes"
            if key not in f:
                continue
            got = bh.let_bucket_boxes(f[key], int(f[f"{system}/c{ci}/bucket_bits"][0]), f[f"{system}/bbox"])
            assert_bits_equal(got, f[f"{system}/c{ci}/boxes"], f"{system} case {ci}")
            seen += 1
    assert seen >= 10


def test_pow5_table_is_generated():
    """The GPU CSV reader's table of 128-bit powers of five is exactly what
    its generator (exact integer arithmetic) writes, and each entry brackets
    5^q as the conversion assumes."""
    import subprocess
    import sys
    from conftest import ROOT
    csrc = ROOT / "barnes-hut_gb300" / "csrc"
    out = subprocess.run([sys.executable, str(csrc / "gen_pow5_table.py")], capture_output=True, text=True,
                         check=True).stdout
    assert out == (csrc / "bh_pow5_table.h").read_text()
    from fractions import Fraction
    sys.path.insert(0, str(csrc))
    import gen_pow5_table as g
    for q in (-342, -300, -28, -27, -1, 0, 1, 27, 55, 56, 200, 308):
        f, s = g.entry(q)
        exact = Fraction(5) ** q
        approx = Fraction(f) * Fraction(2) ** s
        if 0 <= q <= 55:
            assert approx == exact
        elif q > 55:
            assert exact - Fraction(2) ** s < approx <= exact
        else:
            assert exact <= approx < exact + Fraction(2) ** s


def test_model_file_round_trip(bh, tmp_path):
    """bh_mlp_save / bh_mlp_load (host functions): the parameters and scaling
    come back bit for bit; truncated, extended, foreign and missing files are
    refused with a status."""
    rng = np.random.default_rng(4)
    params = rng.normal(size=bh.MLP_PARAMS).astype(np.float32)
    scale = rng.normal(size=bh.MLP_SCALE).astype(np.float32)
    f = tmp_path / "m.bhmlp"
    bh.mlp_save(f, params, scale)
    assert f.stat().st_size == 16 + 4 * (bh.MLP_PARAMS + bh.MLP_SCALE)
    p, s = bh.mlp_load(f)
    assert np.array_equal(p.view(np.uint32), params.view(np.uint32))
    assert np.array_equal(s.view(np.uint32), scale.view(np.uint32))
    data = f.read_bytes()
    for bad in (data[:-4], data + b"\0", b"XXXXXXXX" + data[8:]):
        f.write_bytes(bad)
        with pytest.raises(bh.BhError) as e:
            bh.mlp_load(f)
        assert e.value.status == 1  # BH_ERR_INVALID_ARGUMENT
    with pytest.raises(bh.BhError) as e:
        bh.mlp_load(tmp_path / "missing.bhmlp")
    assert e.value.status == 9  # BH_ERR_IO
    with pytest.raises(ValueError):
        bh.mlp_save(f, params[:10], scale)
