"""readCSV on the GPU (bh_read_csv_gpu, bh_load_csv) against the host
reader (bh_read_csv: std::getline + std::stod, the reference's rules) and
against Python's correctly rounded float(): the same rows, ids, values bit
for bit, body_count limit and warnings.  The comparisons with the
reference's own readCSV are in test_io_pin.py."""
from __future__ import annotations

import random
import sys

import numpy as np
import pytest

from conftest import GOLDEN, assert_bits_equal

sys.path.insert(0, str(GOLDEN))
import csv_cases  # noqa: E402

pytestmark = pytest.mark.gpu

HEADER = csv_cases.HEADER
_num = csv_cases.num
_odd_rows = csv_cases.odd_rows
_rows = csv_cases.rows


def _write(path, rows, crlf=False, final_newline=True):
    csv_cases.write(path, rows, crlf, final_newline)


def _same(a, b):
    for x, y, what in zip(a, b, ("ids", "mass", "pos", "vel")):
        assert_bits_equal(x, y, what)


def test_gpu_reader_matches_host_reader(bh, tmp_path, capfd):
    rng = random.Random(11)
    rows = _rows(rng, 60_000)
    for k, r in enumerate(_odd_rows()):
        rows.insert(100 + 977 * k, r)
    f = tmp_path / "bodies.csv"
    _write(f, rows)
    capfd.readouterr()
    host = bh.read_csv(f)
    host_err = capfd.readouterr().err
    gpu = bh.read_csv_gpu(f)
    gpu_err = capfd.readouterr().err
    assert len(host[0]) == len(rows) - 6  # abc, 1e400, 1e-320, the empty line, ".", the trailing comma
    _same(gpu, host)
    # the same warnings
    assert sorted(set(gpu_err.splitlines())) == sorted(set(host_err.splitlines()))
    assert len(set(host_err.splitlines())) == 6
    # limits: the reference stops after body_count rows
    for lim in (1, 101, 5000):
        _same(bh.read_csv_gpu(f, lim), bh.read_csv(f, lim))


def test_gpu_reader_values_are_correctly_rounded(bh, tmp_path):
    """Every field equals Python's float() of its text (correct rounding),
    including 19-digit mantissas and near-midpoint decimals."""
    rng = random.Random(12)
    fields = [_num(rng) for _ in range(7 * 40_000)]
    fields = [s for s in fields if s.strip() not in ("1e", "1e+", "0e999")]
    fields = fields[: 7 * (len(fields) // 7)]
    rows = [f"{i},b,AST," + ",".join(fields[7 * i: 7 * i + 7]) for i in range(len(fields) // 7)]
    f = tmp_path / "v.csv"
    _write(f, rows)
    ids, mass, pos, vel = bh.read_csv_gpu(f)
    got = np.concatenate([mass[:, None], pos, vel], axis=1).reshape(-1)
    want = np.array([float(s) for s in fields])
    assert_bits_equal(got, want, "values")


@pytest.mark.parametrize("crlf,final_newline", [(True, True), (False, False)])
def test_gpu_reader_line_endings(bh, tmp_path, crlf, final_newline):
    rng = random.Random(13)
    rows = _rows(rng, 2000)
    f = tmp_path / "e.csv"
    _write(f, rows, crlf=crlf, final_newline=final_newline)
    _same(bh.read_csv_gpu(f), bh.read_csv(f))


def test_gpu_reader_empty_and_header_only(bh, tmp_path):
    for text in (b"", HEADER.encode(), (HEADER + "\n").encode()):
        f = tmp_path / "h.csv"
        f.write_bytes(text)
        assert len(bh.read_csv_gpu(f)[0]) == 0
    with pytest.raises(bh.BhError):
        bh.read_csv_gpu(tmp_path / "missing.csv")


def test_load_csv_into_context(bh, tmp_path, golden):
    """bh_load_csv fills the context's state without host arrays: the same
    bodies as the host reader; a context too small is refused."""
    g = golden("synthetic_19054.npz")
    f = tmp_path / "s.csv"
    bh.write_csv(f, g["ids"], g["mass"], g["pos"], g["vel"])
    ids, mass, pos, vel = bh.read_csv(f)
    with bh.Context(len(mass)) as ctx:
        assert ctx.load_csv(f) == len(mass)
        p, v, m, i, a = ctx.get_bodies()
        assert_bits_equal(p, pos, "pos"); assert_bits_equal(v, vel, "vel")
        assert_bits_equal(m, mass, "mass"); assert_bits_equal(i, ids, "ids")
        assert ctx.load_csv(f, 100) == 100
    with bh.Context(1000) as small:
        with pytest.raises(bh.BhError):
            small.load_csv(f)


def test_gpu_reader_streams_large_files(bh, tmp_path):
    """A file of several staging rounds (about 43 MB, beyond the two banks of
    the pinned ring): the same bodies as the host reader, through both entry
    points, with body_count limits that end inside later rounds."""
    rng = np.random.default_rng(14)
    n = 260_000
    ids = np.arange(n, dtype=np.uint64)
    mass = rng.uniform(1e-12, 1e-3, n)
    pos = rng.normal(0.0, 3.0, (n, 3))
    vel = rng.normal(0.0, 1e-2, (n, 3))
    f = tmp_path / "big.csv"
    bh.write_csv(f, ids, mass, pos, vel)
    assert f.stat().st_size > 40 << 20
    host = bh.read_csv(f)
    _same(bh.read_csv_gpu(f), host)
    with bh.Context(n) as ctx:
        for lim in (-1, 200_001):
            k = ctx.load_csv(f, lim)
            assert k == (n if lim < 0 else lim)
            p, v, m, i, _ = ctx.get_bodies()
            assert_bits_equal(p, host[2][:k], "pos"); assert_bits_equal(v, host[3][:k], "vel")
            assert_bits_equal(m, host[1][:k], "mass"); assert_bits_equal(i, host[0][:k], "ids")
