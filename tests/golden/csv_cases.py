"""Seeded state-vector CSV files for the readCSV parity cases, shared by the
fixture generator (make_golden.py) and the tests.  Each file is written from
a seeded ``random.Random``, so the generator and the tests write the same
bytes; the fixtures store each file's SHA-256, and the tests check it first.

Fields take every form the reference's reader (std::getline + std::stod,
src/io.cpp:16-81) meets in practice or must reject: shortest round-trip
decimals, 17-20 significant digits, near-midpoint decimals, integers, hex,
inf/nan, subnormal and overflowing values, short, empty and trailing-comma
rows, extra columns, CRLF line ends and a missing final newline.
"""
from __future__ import annotations

import hashlib
import random
import struct
from decimal import Decimal, getcontext
from pathlib import Path

HEADER = "id,name,class,mass,pos_x,pos_y,pos_z,vel_x,vel_y,vel_z"


def num(rng: random.Random) -> str:
    """A decimal field in one of the forms state-vector files and std::stod
    accept."""
    k = rng.random()
    x = struct.unpack("<d", struct.pack("<Q", rng.getrandbits(64) & ~(0x7FF << 52) |
                                        (rng.randint(1023 - 60, 1023 + 60) << 52)))[0]
    if k < 0.25:
        return repr(x)
    if k < 0.45:
        return f"{x:.18e}"
    if k < 0.55:
        return f"{x:.19g}"
    if k < 0.70:  # 19 significant digits, random exponent
        w = rng.randint(10 ** 18, 10 ** 19 - 1)
        return f"{'-' if rng.random() < 0.5 else ''}{w}e{rng.randint(-60, 40)}"
    if k < 0.80:  # near a rounding boundary: the midpoint of two doubles to 19-20 digits
        getcontext().prec = 50
        b = struct.unpack("<Q", struct.pack("<d", abs(x)))[0]
        mid = (Decimal(abs(x)) + Decimal(struct.unpack("<d", struct.pack("<Q", b + 1))[0])) / 2
        return f"{mid:.19e}" if rng.random() < 0.5 else f"{mid:.18e}"
    if k < 0.85:
        return str(rng.randint(-10 ** 6, 10 ** 6))
    if k < 0.90:
        return rng.choice([" +0.5", ".5", "5.", "1e", "1e+", "-0", "0.000", "  7.25e-3", "3.0\r", "1E5", "0e999"])
    if k < 0.95:  # exact halves and small exact values
        return f"{rng.randint(1, 10 ** 6)}.{rng.choice(['5', '25', '125', '0625'])}"
    return f"{rng.randint(1, 99)}.{rng.randint(0, 10 ** 17):017d}e{rng.randint(-30, 30)}"


def odd_rows() -> list[str]:
    """Rows the device hands to the host or rejects, and getline quirks."""
    return [
        "9,odd,AST,0x1p3,1,2,3,4,5,6",                     # hexadecimal
        "10,odd,AST,inf,1,2,3,4,5,6",                      # inf (valid for std::stod)
        "11,odd,AST,1.2345678901234567890123,1,2,3,4,5,6",  # 23 digits
        "12,odd,AST,1e-320,1,2,3,4,5,6",                   # subnormal (ERANGE -> skipped)
        "13,odd,AST,1e400,1,2,3,4,5,6",                    # overflow: skipped
        "14,odd,AST,abc,1,2,3,4,5,6",                      # no conversion: skipped
        "15,odd,AST,1,2,3,4",                               # short row: fields repeat the last piece
        "16,odd,AST,1,2,3,4,5,6,",                          # trailing comma: an empty field
        "",                                                 # empty line: skipped
        "17,odd,AST,1,2,3,4,5,6,7,extra,columns",           # extra columns are ignored
        "18,odd,AST,nan,1,2,3,4,5,6",                      # nan
        "19,odd,AST,.,1,2,3,4,5,6",                        # no digits: skipped
    ]


def rows(rng: random.Random, n: int) -> list[str]:
    return [f"{i},b{i},AST," + ",".join(num(rng) for _ in range(7)) for i in range(n)]


def write(path: Path, body_rows, crlf=False, final_newline=True) -> str:
    """Writes header + rows; returns the file's SHA-256."""
    nl = "\r\n" if crlf else "\n"
    text = (nl.join([HEADER] + list(body_rows)) + (nl if final_newline else "")).encode()
    Path(path).write_bytes(text)
    return hashlib.sha256(text).hexdigest()


def write_bodies(path: Path, ids, mass, pos, vel) -> str:
    """A state in the state-vector layout readCSV reads, numbers as %.17g
    (round-trip exact); returns the file's SHA-256."""
    lines = [HEADER]
    for k in range(len(mass)):
        vals = [mass[k], *pos[k], *vel[k]]
        lines.append(f"{int(ids[k])},b{int(ids[k])},AST," + ",".join("%.17g" % v for v in vals))
    data = ("\n".join(lines) + "\n").encode()
    Path(path).write_bytes(data)
    return hashlib.sha256(data).hexdigest()


def hostile(n: int, seed: int, spacing: int = 977) -> list[str]:
    """n seeded rows with the odd rows inserted from row 100 on, `spacing`
    apart."""
    body = rows(random.Random(seed), n)
    for k, r in enumerate(odd_rows()):
        body.insert(min(len(body), 100 + spacing * k), r)
    return body


# The cases pinned against the reference's readCSV: name -> (rows, crlf,
# final_newline, body_count limits).  The first is also the large-file case
# of the GPU reader's tests.
def cases() -> dict:
    return {
        "mixed_60k": (lambda: hostile(60_000, 11), False, True, (-1, 1, 101, 5000)),
        "mixed_3k": (lambda: hostile(3_000, 21, spacing=211), False, True, (-1, 7)),
        "crlf": (lambda: rows(random.Random(13), 2000), True, True, (-1,)),
        "no_final_newline": (lambda: rows(random.Random(13), 2000), False, False, (-1,)),
        "short_rows": (lambda: ["0,a,b,5.0,1,2,3,4,5", "1,a,b,7,8", "2,a,b", "3,a,b,1,2,3,4,5,6"], False, True,
                       (-1,)),
    }
