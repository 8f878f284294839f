"""ctypes front end of the oracle (TEST INFRASTRUCTURE ONLY).

Two libraries with the same calling conventions:

* ``Oracle("port")``      -- oracle/_build/libbhoracle.so, the C restatement
                              (bh_oracle.c) of the reference's path; builds on
                              any host with gcc (``make -C oracle``).
* ``Oracle("reference")`` -- oracle/_ref/libbhref.so, the reference's own
                              sources compiled by ``make -C oracle ref``
                              (only where the reference checkout exists).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline and
reference legs use this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_LIB = HERE / "_build" / "libbhoracle.so"
REF_LIB = HERE / "_ref" / "libbhref.so"
# The reference checkout: $BH_REFERENCE_DIR, else its usual location.
REF_SRC = Path(os.environ.get("BH_REFERENCE_DIR") or "/root/reference")

_P = C.c_void_p
_I64 = C.c_int64
_D = C.c_double


def build_port() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    return PORT_LIB


def build_reference() -> Path | None:
    """Compiles the reference's sources when the checkout is present."""
    if not (REF_SRC / "src" / "traversal.cpp").exists():
        return REF_LIB if REF_LIB.exists() else None
    subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF={REF_SRC}"], check=True)
    return REF_LIB


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Oracle:
    def __init__(self, kind: str = "port"):
        self.kind = kind
        if kind == "port":
            path = PORT_LIB if PORT_LIB.exists() else build_port()
            pre = "orc_"
        elif kind == "reference":
            path = REF_LIB
            if not path.exists():
                raise FileNotFoundError(f"{path} not built (make -C oracle ref)")
            pre = "ref_"
        else:
            raise ValueError(kind)
        self.lib = C.CDLL(str(path))
        self.pre = pre
        L, p = self.lib, pre

        def f(name, res, args):
            fn = getattr(L, p + name)
            fn.restype = res
            fn.argtypes = args
            return fn

        if kind == "port":
            self._bbox = f("bbox", None, [_P, _I64, _P])
            self._keys = f("keys", None, [_P, _I64, _P, _P])
            self._sort = f("sort_bodies", C.c_int, [_I64, _P, _P, _P, _P, _P, _P])
            self._build = f("build_tree", _P, [_I64, _P, _P, _P, C.c_int])
            self._size = f("tree_size", _I64, [_P])
            self._records = f("tree_records", C.c_int, [_P, _P, _P, _P, _P])
            self._free = f("tree_free", None, [_P])
            self._accel = f("accelerations", C.c_int, [_P, _I64, _P, _P, _D, _D, _D, _P, _P, _P])
            self._gen = f("generate_system", C.c_int, [C.c_uint64, _I64, _D, _D, _P, _P, _P, _P])
            self._accel_at = f("accelerations_at", C.c_int, [_P, _I64, _P, _P, _P, _D, _D, _D, _P, _P, _P])
            self._sim = f("simulate", C.c_int, [_I64, _P, _P, _P, _P, _P, _D, _D, _D, _I64, _P, _P])
            self._kepler = f("kepler_to_cartesian", None, [_P, _I64, _P])
            self._direct = f("direct_sum", None, [_I64, _P, _P, _I64, _P, _D, _P])
            self._inv = f("invariants", None, [_I64, _P, _P, _P, _D, _P])
            self._threads = f("num_threads", C.c_int, [])
            self._let = f("let_export", _I64, [_P, _P, _I64, _P, _D, C.c_int, _P, _P, _P, _P, _I64])
            self._pseudo = f("pseudo_tree", _P, [_P, _P, _P, _P, _I64])
            self._letacc = f("let_accelerations", C.c_int, [_P, _P, _P, _P, _P, _I64, _I64, _P, _P, _D, _D, _D, _P,
                                                             C.c_int, _P])
        else:
            self._bbox = f("compute_local_bbox", None, [_P, _I64, _P])
            self._keys = f("generate_morton_codes", None, [_P, _I64, _P, _P])
            self._sort = f("sort_bodies", None, [_I64, _P, _P, _P, _P, _P])
            self._build = f("build_tree", _P, [_I64, _P, _P, _P, C.c_int])
            self._size = f("tree_size", _I64, [_P])
            self._records = f("tree_records", None, [_P, _P, _P, _P, _P])
            self._free = f("tree_free", None, [_P])
            self._accel = f("compute_accelerations", None, [_P, _I64, _P, _P, _D, _D, _D, _P, _P])
            self._sim = f("simulate", None, [_I64, _P, _P, _P, _P, _P, _D, _D, _D, _I64, _P, _P])
            self._kepler = f("kepler_to_cartesian", None, [_P, _I64, _P])
            self._let = f("let_export", _I64, [_P, _P, _I64, _P, _D, C.c_int, _P, _P, _P, _P, _I64])
            self._pseudo = f("pseudo_tree", _P, [_P, _P, _P, _P, _I64])
            self._letacc = f("let_accelerations", None, [_P, _P, _P, _P, _P, _I64, _I64, _P, _P, _D, _D, _D, _P,
                                                          C.c_int, _P])
            # src/io.cpp through oracle/ref_io_harness.cpp
            self._read_csv = f("read_csv", _I64, [C.c_char_p, C.c_int, _P, _P, _P, _P, _I64])
            self._snapshot = f("write_snapshot", None, [C.c_int, C.c_int, _I64, _P, _P, _P, _P, _P, C.c_char_p])
            self._pvd = f("update_pvd", None, [C.c_int, C.POINTER(C.c_char_p), C.c_int, C.c_int, _D, C.c_char_p])
            self._save_ref = f("save_reference_csv", None, [C.c_char_p, _I64, _P, _P])
            self._load_ref = f("load_reference_csv", C.c_int, [C.c_char_p, C.c_int, _P])
            self._dist = f("compute_distance_sum", _D, [_I64, _P, _P, _I64, _P])
            self._cli = f("run_cli", C.c_int, [C.c_int, C.POINTER(C.c_char_p), _P, _P, _P, _P])

    # -- stages ---------------------------------------------------------
    def bbox(self, pos) -> np.ndarray:
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        out = np.empty(6)
        self._bbox(_ptr(pos), pos.shape[0], _ptr(out))
        return out

    def keys(self, pos, bbox) -> np.ndarray:
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        bb = np.ascontiguousarray(bbox, np.float64)
        out = np.empty(pos.shape[0], np.uint64)
        self._keys(_ptr(pos), pos.shape[0], _ptr(bb), _ptr(out))
        return out

    def sort(self, keys, pos, mass, vel, ids):
        """Sorted copies (keys, pos, mass, vel, ids[, perm for the port])."""
        k = np.array(keys, np.uint64); p = np.array(pos, np.float64).reshape(-1, 3)
        m = np.array(mass, np.float64); v = np.array(vel, np.float64).reshape(-1, 3)
        i = np.array(ids, np.uint64)
        if self.kind == "port":
            perm = np.empty(len(k), np.int64)
            self._sort(len(k), _ptr(k), _ptr(p), _ptr(m), _ptr(v), _ptr(i), _ptr(perm))
            return k, p, m, v, i, perm
        self._sort(len(k), _ptr(k), _ptr(p), _ptr(m), _ptr(v), _ptr(i))
        return k, p, m, v, i, None

    def tree(self, keys, pos, mass, merge=True):
        k = np.ascontiguousarray(keys, np.uint64)
        p = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        m = np.ascontiguousarray(mass, np.float64)
        h = self._build(len(k), _ptr(k), _ptr(p), _ptr(m), 1 if merge else 0)
        if not h:
            raise MemoryError("oracle tree build failed")
        return OracleTree(self, h)

    def accelerations(self, tree, keys, pos, theta, G, soft2, bbox, count=False):
        k = np.ascontiguousarray(keys, np.uint64)
        p = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        bb = np.ascontiguousarray(bbox, np.float64)
        acc = np.empty((len(k), 3))
        if self.kind == "port":
            cnt = np.empty(len(k), np.int64) if count else None
            rc = self._accel(tree.h, len(k), _ptr(k), _ptr(p), theta, G, soft2, _ptr(bb), _ptr(acc), _ptr(cnt))
            if rc:
                raise RuntimeError(f"oracle traversal failed: {rc}")
            return (acc, cnt) if count else acc
        self._accel(tree.h, len(k), _ptr(k), _ptr(p), theta, G, soft2, _ptr(bb), _ptr(acc))
        return acc

    def accelerations_at(self, tree, keys, pos, targets, theta, G, soft2, bbox):
        """computeAccelerations' walk for the bodies `targets` (indices into
        keys/pos) only: (acc (k, 3), interactions (k,)).  Port only."""
        k = np.ascontiguousarray(keys, np.uint64)
        p = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        t = np.ascontiguousarray(targets, np.int64)
        if len(t) and (t.min() < 0 or t.max() >= len(k)):
            raise IndexError("target out of range")
        bb = np.ascontiguousarray(bbox, np.float64)
        acc = np.empty((len(t), 3))
        cnt = np.empty(len(t), np.int64)
        rc = self._accel_at(tree.h, len(t), _ptr(t), _ptr(k), _ptr(p), theta, G, soft2, _ptr(bb), _ptr(acc), _ptr(cnt))
        if rc:
            raise RuntimeError(f"oracle traversal failed: {rc}")
        return acc, cnt

    def let_export(self, tree, boxes, bbox, theta2, max_depth=21):
        """createInteractionListForRank (src/exchange.cpp:117-179) on `tree`:
        the exported cells (prefix, depth, mass, com) sorted by (depth, prefix)."""
        bx = np.ascontiguousarray(boxes, np.float64).reshape(-1, 6)
        bb = np.ascontiguousarray(bbox, np.float64)
        cap = len(tree)
        p = np.empty(cap, np.uint64); d = np.empty(cap, np.uint8); m = np.empty(cap); c = np.empty((cap, 3))
        k = int(self._let(tree.h, _ptr(bx), len(bx), _ptr(bb), theta2, int(max_depth), _ptr(p), _ptr(d), _ptr(m),
                          _ptr(c), cap))
        o = np.lexsort((p[:k], d[:k]))
        return p[:k][o], d[:k][o], m[:k][o], c[:k][o]

    def pseudo_tree(self, prefix, depth, mass, com) -> "OracleTree":
        """buildTreeFromPseudoLeaves (src/linear_octree.cpp:242-322) over
        NodeRecords; read the map back with .records()."""
        p = np.ascontiguousarray(prefix, np.uint64); d = np.ascontiguousarray(depth, np.uint8)
        m = np.ascontiguousarray(mass, np.float64); c = np.ascontiguousarray(com, np.float64).reshape(-1, 3)
        h = self._pseudo(_ptr(p), _ptr(d), _ptr(m), _ptr(c), len(p))
        if not h:
            raise MemoryError("pseudo_tree")
        return OracleTree(self, h)

    def let_accelerations(self, tree, records, keys, pos, theta, G, bbox, soft2=0.0, direct=False):
        """computeAccelerationsWithLET (direct=False) or
        computeAccelerationsWithRemoteDirectSum (direct=True): local `tree`
        (unchanged), received `records` = (prefix, depth, mass, com), bodies
        with `keys` and `pos`."""
        p = np.ascontiguousarray(records[0], np.uint64); d = np.ascontiguousarray(records[1], np.uint8)
        m = np.ascontiguousarray(records[2], np.float64)
        c = np.ascontiguousarray(records[3], np.float64).reshape(-1, 3)
        k = np.ascontiguousarray(keys, np.uint64); x = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        bb = np.ascontiguousarray(bbox, np.float64)
        out = np.empty((len(k), 3))
        rc = self._letacc(tree.h, _ptr(p), _ptr(d), _ptr(m), _ptr(c), len(m), len(k), _ptr(k), _ptr(x), theta, G,
                          soft2, _ptr(bb), int(direct), _ptr(out))
        if rc:
            raise RuntimeError(f"oracle let_accelerations failed ({rc})")
        return out

    def simulate(self, pos, vel, mass, ids, dt, theta, G, nsteps, t=0.0, acc=None):
        """Runs the step loop; returns (pos, vel, mass, ids, acc, t, phase_s)."""
        p = np.array(pos, np.float64).reshape(-1, 3); v = np.array(vel, np.float64).reshape(-1, 3)
        m = np.array(mass, np.float64); i = np.array(ids, np.uint64)
        a = np.zeros_like(p) if acc is None else np.array(acc, np.float64).reshape(-1, 3)
        tt = _D(t)
        ph = np.zeros(7)
        rc = self._sim(len(m), _ptr(p), _ptr(v), _ptr(m), _ptr(i), _ptr(a), dt, theta, G, int(nsteps),
                       C.byref(tt), _ptr(ph))
        if self.kind == "port" and rc:
            raise RuntimeError(f"oracle simulate failed: {rc}")
        return p, v, m, i, a, tt.value, ph

    def kepler(self, el) -> np.ndarray:
        e = np.ascontiguousarray(el, np.float64).reshape(-1, 8)
        out = np.empty((e.shape[0], 6))
        self._kepler(_ptr(e), e.shape[0], _ptr(out))
        return out

    def direct_sum(self, pos, mass, targets, G) -> np.ndarray:
        p = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        m = np.ascontiguousarray(mass, np.float64)
        t = np.ascontiguousarray(targets, np.int64)
        out = np.empty((len(t), 3))
        self._direct(len(m), _ptr(p), _ptr(m), len(t), _ptr(t), G, _ptr(out))
        return out

    def invariants(self, pos, vel, mass, G) -> np.ndarray:
        p = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        v = np.ascontiguousarray(vel, np.float64).reshape(-1, 3)
        m = np.ascontiguousarray(mass, np.float64)
        out = np.empty(9)
        self._inv(len(m), _ptr(p), _ptr(v), _ptr(m), G, _ptr(out))
        return out

    def generate_system(self, seed, n, frac_outer=0.0, frac_trojan=0.0):
        """The seeded synthetic solar system (port only): (pos, vel, mass,
        ids), the engine generator's draws restated."""
        pos = np.empty((n, 3)); vel = np.empty((n, 3)); mass = np.empty(n); ids = np.empty(n, np.uint64)
        if self._gen(int(seed), int(n), float(frac_outer), float(frac_trojan), _ptr(pos), _ptr(vel), _ptr(mass),
                     _ptr(ids)):
            raise ValueError("generate_system: need n >= 9 and fractions in [0, 1]")
        return pos, vel, mass, ids

    def threads(self) -> int:
        return int(self._threads()) if self.kind == "port" else -1

    # -- the reference's I/O (src/io.cpp; reference kind only) -----------
    def read_csv(self, path, body_count=-1, cap=None):
        """readCSV (src/io.cpp:16-81): (ids, mass, pos, vel).  `cap` bounds
        the rows copied (default: the file's line count)."""
        path = str(path)
        if cap is None:
            with open(path, "rb") as fh:
                cap = fh.read().count(b"\n") + 1
        ids = np.empty(cap, np.uint64); mass = np.empty(cap); pos = np.empty((cap, 3)); vel = np.empty((cap, 3))
        n = int(self._read_csv(path.encode(), int(body_count), _ptr(ids), _ptr(mass), _ptr(pos), _ptr(vel), cap))
        if n < 0:
            raise FileNotFoundError(path)
        k = min(n, cap)
        return ids[:k], mass[:k], pos[:k], vel[:k]

    def write_snapshot(self, rank, vs_counter, ids, mass, pos, vel, acc, vs_dir):
        """writeSnapshot (src/io.cpp:84-232) into <vs_dir>/<rank>/sim.<k>.vtp."""
        i = np.ascontiguousarray(ids, np.uint64); m = np.ascontiguousarray(mass, np.float64)
        p, v, a = (np.ascontiguousarray(x, np.float64).reshape(-1, 3) for x in (pos, vel, acc))
        self._snapshot(int(rank), int(vs_counter), len(m), _ptr(i), _ptr(m), _ptr(p), _ptr(v), _ptr(a),
                       str(vs_dir).encode())

    @staticmethod
    def _argv(args):
        arr = (C.c_char_p * (len(args) + 1))(*[a.encode() for a in ["simulate", *args]])
        return len(args) + 1, arr

    def update_pvd(self, args, size, vs_counter, t, vs_dir):
        """updatePVDFile (src/io.cpp:234-298) for the command line `args`."""
        argc, argv = self._argv(args)
        self._pvd(argc, argv, int(size), int(vs_counter), float(t), str(vs_dir).encode())

    def save_reference_csv(self, d, pos, ids):
        p = np.ascontiguousarray(pos, np.float64).reshape(-1, 3); i = np.ascontiguousarray(ids, np.uint64)
        self._save_ref(str(d).encode(), len(i), _ptr(p), _ptr(i))

    def load_reference_csv(self, d, n):
        out = np.empty((n, 3))
        if self._load_ref(str(d).encode(), int(n), _ptr(out)):
            raise FileNotFoundError(f"{d}/final_ref.csv")
        return out

    def distance_sum(self, pos, ids, ref_pos) -> float:
        p = np.ascontiguousarray(pos, np.float64).reshape(-1, 3); i = np.ascontiguousarray(ids, np.uint64)
        r = np.ascontiguousarray(ref_pos, np.float64).reshape(-1, 3)
        return float(self._dist(len(i), _ptr(p), _ptr(i), len(r), _ptr(r)))

    def run_cli(self, args):
        """The reference driver (src/main.cpp) on one rank for the tree force
        path with command line `args`, in the current directory: returns
        (SUMMED_DIST_ERROR, bodies, steps, frames)."""
        argc, argv = self._argv(args)
        s = _D(); n = _I64(); k = _I64(); fr = _I64()
        if self._cli(argc, argv, C.byref(s), C.byref(n), C.byref(k), C.byref(fr)):
            raise FileNotFoundError("input file")
        return s.value, n.value, k.value, fr.value


class OracleTree:
    def __init__(self, oracle: Oracle, h):
        self.o = oracle
        self.h = h

    def __len__(self):
        return int(self.o._size(self.h))

    def records(self):
        n = len(self)
        prefix = np.empty(n, np.uint64); depth = np.empty(n, np.uint8); mass = np.empty(n)
        com = np.empty((n, 3))
        self.o._records(self.h, _ptr(prefix), _ptr(depth), _ptr(mass), _ptr(com))
        return prefix, depth, mass, com

    def close(self):
        if self.h:
            self.o._free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
