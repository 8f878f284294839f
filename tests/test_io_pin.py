"""The I/O of the path pinned to the reference's own io.cpp.

tests/golden/io.npz was written by the reference's src/io.cpp (and its
vendored tinyxml2), compiled unmodified with the oracle's recipe
(make_golden.py `io`):

* readCSV (io.cpp:16-81) on the seeded CSV files of csv_cases.py: row
  counts, the parsed arrays (digests; in full for the small files), the
  body_count limits and the warnings it prints;
* writeSnapshot (io.cpp:84-232) and updatePVDFile (io.cpp:234-298): the
  bytes of the files;
* the reference driver (main.cpp:44-345 on one rank, tree path) on a
  1,000-body CSV: every snapshot and .pvd file of its schedule
  (main.cpp:283-320), final_ref.csv of a -r run (saveReferenceCSV,
  io.cpp:716-722) and SUMMED_DIST_ERROR of a rerun against it
  (loadReferenceCSV + computeDistanceSum, io.cpp:725-779).

The host functions (bh_read_csv, bh_write_vtp) are compared here on the
CPU; the GPU reader, bh_load_csv and the simulate driver in the gpu tests.
Every comparison is bit- or byte-exact."""
from __future__ import annotations

import hashlib
import subprocess
import sys

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, assert_bits_equal

sys.path.insert(0, str(GOLDEN))
import csv_cases  # noqa: E402

SIMULATE = ROOT / "barnes-hut_gb300" / "_build" / "simulate"


@pytest.fixture(scope="module")
def io():
    return np.load(GOLDEN / "io.npz", allow_pickle=False)


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def _csv_files(tmp_path, io):
    """Writes each case's file and checks it is the file the fixture was
    made from; yields (name, path, limits)."""
    for name, (make_rows, crlf, final_nl, limits) in csv_cases.cases().items():
        f = tmp_path / f"{name}.csv"
        assert csv_cases.write(f, make_rows(), crlf, final_nl) == str(io[f"csv/{name}/sha256"][0]), name
        yield name, f, limits


def _check_read(io, key, got, what):
    ids, mass, pos, vel = got
    assert len(mass) == int(io[f"{key}/n"][0]), f"{what}: row count"
    if f"{key}/mass" in io:
        for a, k in ((ids, "ids"), (mass, "mass"), (pos, "pos"), (vel, "vel")):
            assert_bits_equal(a, io[f"{key}/{k}"], f"{what} {k}")
    assert digest(np.asarray(ids, np.uint64), mass, pos, vel) == str(io[f"{key}/digest"][0]), what


def _warnings(err: str) -> list[str]:
    return [ln for ln in err.splitlines() if ln.startswith("Warning:")]


def test_host_reader_matches_reference_readcsv(bh, tmp_path, capfd, io):
    """bh_read_csv: the same rows, values, ids, limits and warnings (in
    order) as readCSV."""
    for name, f, limits in _csv_files(tmp_path, io):
        for lim in limits:
            capfd.readouterr()
            got = bh.read_csv(f, lim)
            err = capfd.readouterr().err
            key = f"csv/{name}/lim{lim}"
            _check_read(io, key, got, f"{name} limit {lim}")
            assert _warnings(err) == _warnings(str(io[f"{key}/warnings"][0])), f"{name} limit {lim} warnings"
    for name in ("empty", "header_only", "header_newline"):
        f = tmp_path / f"{name}.csv"
        f.write_bytes({"empty": b"", "header_only": csv_cases.HEADER.encode(),
                       "header_newline": (csv_cases.HEADER + "\n").encode()}[name])
        assert len(bh.read_csv(f)[1]) == int(io[f"csv/{name}/n"][0]) == 0


def test_vtp_writer_matches_reference_bytes(bh, tmp_path, io):
    """bh_write_vtp writes writeSnapshot's bytes (rank 3; signed zeros,
    inf/nan, a subnormal, an overflowing |a|, 40-bit ids); an empty state
    writes no file, as in the reference."""
    path = tmp_path / "sim.2.vtp"
    bh.write_vtp(path, io["vtp/ids"], io["vtp/mass"], io["vtp/pos"], io["vtp/vel"], io["vtp/acc"], rank=3)
    assert path.read_bytes() == io["vtp/bytes"].tobytes()
    empty = tmp_path / "empty.vtp"
    e = np.empty((0, 3))
    bh.write_vtp(empty, np.empty(0, np.uint64), np.empty(0), e, e, e)
    assert empty.exists() == bool(io["vtp/empty_writes_file"][0]) is False


def test_scenario1_reader_matches_reference():
    """The reference's own scenario-1 file (where the checkout is present):
    bh_read_csv gives the arrays the reference's readCSV gave."""
    import importlib
    import json
    from oracle.oracle import REF_SRC
    csv = REF_SRC / "data" / "state_vectors_csvs" / "scenario1_19054.csv"
    if not csv.exists():
        pytest.skip("reference checkout not present")
    bh = importlib.import_module("barnes-hut_gb300")
    ids, mass, pos, vel = bh.read_csv(csv)
    info = json.loads((GOLDEN / "scenario1.json").read_text())
    assert len(mass) == info["n"] and digest(pos, vel, mass, ids) == info["input_digest"]


@pytest.mark.gpu
def test_gpu_reader_matches_reference_readcsv(bh, tmp_path, capfd, io):
    """bh_read_csv_gpu: readCSV's rows, values, ids and limits bit for bit,
    and the same warnings (the two-pass reader may print one twice)."""
    for name, f, limits in _csv_files(tmp_path, io):
        for lim in limits:
            capfd.readouterr()
            got = bh.read_csv_gpu(f, lim)
            err = capfd.readouterr().err
            key = f"csv/{name}/lim{lim}"
            _check_read(io, key, got, f"{name} limit {lim}")
            assert set(_warnings(err)) == set(_warnings(str(io[f"{key}/warnings"][0]))), f"{name} warnings"


@pytest.mark.gpu
def test_load_csv_matches_reference_readcsv(bh, tmp_path, io):
    """bh_load_csv straight into the device state: readCSV's bodies."""
    files = {name: (f, limits) for name, f, limits in _csv_files(tmp_path, io)}
    for name in ("mixed_3k", "mixed_60k", "crlf"):
        f, limits = files[name]
        with bh.Context(int(io[f"csv/{name}/lim-1/n"][0])) as ctx:
            for lim in limits:
                k = ctx.load_csv(f, lim)
                p, v, m, i, _ = ctx.get_bodies()
                _check_read(io, f"csv/{name}/lim{lim}", (i, m, p, v), f"{name} limit {lim}")
                assert k == len(m)


def _run_simulate(args, cwd):
    r = subprocess.run([str(SIMULATE), *args], capture_output=True, text=True, cwd=cwd)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = {ln.split()[0]: ln for ln in r.stdout.splitlines() if ln.strip()}
    return r.stdout, lines


@pytest.mark.gpu
def test_simulate_matches_reference_driver_files(bh, tmp_path, io, golden):
    """simulate on the reference driver's command lines, in order in one
    directory: the same snapshot and .pvd files byte for byte (frame schedule,
    file names from -f/--dt/--tend/--theta/-b/--fc, number formatting), the
    same final_ref.csv after -r, and the rerun's SUMMED_DIST_ERROR equal to
    computeDistanceSum's to the last bit."""
    if not SIMULATE.exists():
        pytest.skip("simulate not built (run build())")
    g = golden("synthetic_1000.npz")
    sha = csv_cases.write_bodies(tmp_path / "bodies.csv", g["ids"], g["mass"], g["pos"], g["vel"])
    assert sha == str(io["cli/bodies_sha256"][0])
    for name in ("frames", "limit", "reference", "rerun"):
        args = [str(a) for a in io[f"cli/{name}/args"]]
        out, lines = _run_simulate(args, tmp_path)
        n, steps, frames = (int(x) for x in io[f"cli/{name}/counts"])
        assert f"Loaded {n} bodies" in out
        assert out.count("Saved frame") == frames
        odir = tmp_path / args[args.index("-o") + 1]
        files = sorted(str(p.relative_to(odir)) for p in odir.rglob("*") if p.is_file())
        assert files == [str(x) for x in io[f"cli/{name}/files"]], name
        for fname, want in zip(files, io[f"cli/{name}/sha256"]):
            data = (odir / fname).read_bytes()
            key = f"cli/{name}/bytes/{fname}"
            if key in io:
                assert data == io[key].tobytes(), f"{name}: {fname}"
            assert hashlib.sha256(data).hexdigest() == str(want), f"{name}: {fname}"
        summed = float(io[f"cli/{name}/summed"][0])
        assert float(lines["SUMMED_DIST_ERROR_FULL"].split()[1]) == summed, name
        assert lines["SUMMED_DIST_ERROR"] == f"SUMMED_DIST_ERROR   {summed:.4f}"
        if name == "reference":
            assert (tmp_path / "reference" / "final_ref.csv").read_bytes() == io["cli/final_ref_csv"].tobytes()
    assert float(io["cli/rerun/summed"][0]) > 0.0


def test_reference_csv_loader_fixture_is_consistent(io):
    """The fixture's loadReferenceCSV result is the -r file's text read back
    (6 significant digits), and its distance sum over a reversed body order
    equals the sum recomputed here in the reference's order."""
    text = io["cli/final_ref_csv"].tobytes().decode().splitlines()
    assert text[0] == "id,x,y,z"
    rp = np.zeros_like(io["cli/final_ref_loaded"])
    for ln in text[1:]:
        f = ln.split(",")
        rp[int(f[0])] = [float(x) for x in f[1:4]]
    assert_bits_equal(rp, io["cli/final_ref_loaded"], "loadReferenceCSV")
