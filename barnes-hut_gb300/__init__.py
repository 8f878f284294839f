"""GB300 Barnes-Hut engine: Python host bindings over libbh_gpu.so (C ABI).

The compute path is the CUDA library ``_build/libbh_gpu.so`` (built by
``build.py``); this module only marshals numpy arrays through ctypes.  There is
no CPU fallback: every compute call raises if the library is missing or no
GPU is present.

Reference-shaped entry points (YonatanGM/Barnes-Hut, single-rank ``--fc tree``):

=========================  ===============================================
``compute_local_bbox``     compute_local_bbox, src/bounding_box.cpp:23-44
``generateMortonCodes``    generateMortonCodes, src/morton_keys.cpp:65-98
``sortBodiesByMortonKey``  sortBodiesByMortonKey, include/utility.h:23-52
``buildOctreeBottomUp``    buildOctreeBottomUp + exchangeFullTrees merge,
                           src/linear_octree.cpp:13-107, 178-204
``computeAccelerations``   computeAccelerations, src/traversal.cpp:13-103
``Simulation.step``        the step loop of src/main.cpp:191-282
``read_csv``               readCSV, src/io.cpp:16-81
``kepler_to_cartesian``    convertKeplerToCartesian,
                           src/kepler_to_cartesian.cpp:13-107
=========================  ===============================================

Arrays: positions/velocities/accelerations are (n, 3) float64 (the
reference's Vec3 AoS), masses (n,) float64, ids and keys (n,) uint64.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_build" / "libbh_gpu.so"

G_DEFAULT = 1.48812e-34  # AU^3 kg^-1 day^-2 (src/main.cpp:174)
THETA_DEFAULT = 1.05     # src/main.cpp:61
MAX_DEPTH = 21
NUM_MASSIVE = 9

MODE_PLAIN_FP64 = 0
MODE_FP64_LIST = 1
MODE_FP32_FAR = 2
MODE_LEARNED = 3
MODE_FP32_GROUP = 4

STATUS = {
    0: "BH_OK", 1: "BH_ERR_INVALID_ARGUMENT", 2: "BH_ERR_CUDA", 3: "BH_ERR_OUT_OF_MEMORY",
    4: "BH_ERR_CAPACITY", 5: "BH_ERR_OVERFLOW", 6: "BH_ERR_TIMEOUT", 7: "BH_ERR_NONFINITE",
    8: "BH_ERR_STATE", 9: "BH_ERR_IO", 10: "BH_ERR_NO_DEVICE",
}


class BhError(RuntimeError):
    """A non-zero status from libbh_gpu.so, with the library's message."""

    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"{STATUS.get(status, status)}: {message}")


_lib = None
_P = C.c_void_p
_I64 = C.c_int64
_D = C.c_double


def _sig(lib):
    f = {}
    f["bh_last_error"] = (C.c_char_p, [])
    f["bh_status_string"] = (C.c_char_p, [C.c_int])
    f["bh_api_version"] = (C.c_int, [])
    f["bh_context_create"] = (C.c_int, [_I64, C.c_int, C.POINTER(_P)])
    f["bh_context_destroy"] = (C.c_int, [_P])
    f["bh_context_sync"] = (C.c_int, [_P])
    f["bh_context_stream"] = (C.c_int, [_P, C.POINTER(_P)])
    f["bh_set_bodies"] = (C.c_int, [_P, _I64, _P, _P, _P, _P])
    f["bh_get_bodies"] = (C.c_int, [_P, _P, _P, _P, _P, _P])
    f["bh_set_accelerations"] = (C.c_int, [_P, _P])
    f["bh_num_bodies"] = (C.c_int, [_P, C.POINTER(_I64)])
    f["bh_compute_bbox"] = (C.c_int, [_P, _P])
    f["bh_compute_keys"] = (C.c_int, [_P, _P])
    f["bh_set_bbox"] = (C.c_int, [_P, _P])
    f["bh_sort_bodies"] = (C.c_int, [_P, _P])
    f["bh_build_tree"] = (C.c_int, [_P])
    f["bh_build_tree_options"] = (C.c_int, [_P, C.c_int])
    f["bh_tree_info"] = (C.c_int, [_P, C.POINTER(_I64), C.POINTER(_I64), C.POINTER(_I64)])
    f["bh_export_tree"] = (C.c_int, [_P, _P, _P, _P, _P])
    f["bh_compute_accelerations"] = (C.c_int, [_P, _D, _D, _D, C.c_int, _P])
    f["bh_interaction_count"] = (C.c_int, [_P, C.POINTER(_I64)])
    f["bh_interaction_counts"] = (C.c_int, [_P, _P])
    f["bh_step"] = (C.c_int, [_P, _D, _D, _D, _I64, C.c_int, C.POINTER(_D)])
    f["bh_step_host"] = (C.c_int, [_P, _I64, _P, _P, _P, _P, _P, _D, _D, _D, _I64, C.c_int, C.POINTER(_D)])
    f["bh_set_profiling"] = (C.c_int, [_P, C.c_int])
    f["bh_phase_times"] = (C.c_int, [_P, _P, C.POINTER(_I64)])
    f["bh_measure_fma_peak"] = (C.c_int, [_P, C.c_int, C.POINTER(_D)])
    f["bh_direct_sum"] = (C.c_int, [_P, _I64, _P, _D, _P])
    f["bh_invariants"] = (C.c_int, [_P, _D, _D, _P])
    f["bh_tree_spread"] = (C.c_int, [_P, _P])
    f["bh_set_step_graphs"] = (C.c_int, [_P, C.c_int])
    f["bh_kepler_to_cartesian_gpu"] = (C.c_int, [_P, _I64, _P])
    f["bh_write_vtp"] = (C.c_int, [C.c_char_p, C.c_int, _I64, _P, _P, _P, _P, _P])
    f["bh_selftest"] = (C.c_int, [C.c_int, _I64, C.c_uint64, C.POINTER(_I64)])
    f["bh_tree_slots"] = (C.c_int, [_P, _P, _P])
    f["bh_let_export"] = (C.c_int, [_P, _P, _I64, _P, _D, C.c_int, _I64, _P, _P, _P, _P, C.POINTER(_I64)])
    f["bh_let_bucket_boxes"] = (C.c_int, [_P, _I64, C.c_int, _P, _P])
    f["bh_pseudo_leaf_tree"] = (C.c_int, [_P, _P, _P, _P, _P, _I64, _I64, _P, _P, _P, _P, C.POINTER(_I64)])
    f["bh_let_accelerations"] = (C.c_int, [_P, _P, _P, _P, _P, _I64, _D, _D, _D, _P])
    f["bh_let_direct_accelerations"] = (C.c_int, [_P, _P, _P, _P, _P, _I64, _D, _D, _D, _P])
    f["bh_mlp_gradient"] = (C.c_int, [_P, _P, _P, _I64, _P, _P])
    f["bh_mlp_train"] = (C.c_int, [_P, _P, _I64, C.c_int, C.c_int, C.c_float, C.c_uint64, _P, _P, _P])
    f["bh_mlp_predict"] = (C.c_int, [_P, _P, _P, _I64, _P, _P])
    f["bh_learned_collect"] = (C.c_int, [_P, _D, _D, _D, _D, _I64, _P, _P, C.POINTER(_I64)])
    f["bh_learned_set_model"] = (C.c_int, [_P, _P, _P, _D, _D])
    f["bh_learned_stats"] = (C.c_int, [_P, _P])
    f["bh_learned_set_criterion"] = (C.c_int, [_P, _D, _D])
    f["bh_mlp_save"] = (C.c_int, [C.c_char_p, _P, _P])
    f["bh_mlp_load"] = (C.c_int, [C.c_char_p, _P, _P])
    f["bh_compute_local_bbox"] = (C.c_int, [_P, _I64, _P])
    f["bh_generate_morton_codes"] = (C.c_int, [_P, _I64, _P, _P])
    f["bh_sort_bodies_by_morton_key"] = (C.c_int, [_I64, _P, _P, _P, _P, _P])
    f["bh_kepler_to_cartesian"] = (C.c_int, [_P, _I64, _P])
    f["bh_generate_system"] = (C.c_int, [C.c_uint64, _I64, _D, _D, _P, _P, _P, _P])
    f["bh_read_csv"] = (C.c_int, [C.c_char_p, _I64, C.POINTER(_I64), _P, _P, _P, _P])
    f["bh_write_csv"] = (C.c_int, [C.c_char_p, _I64, _P, _P, _P, _P])
    f["bh_read_csv_gpu"] = (C.c_int, [C.c_char_p, _I64, C.POINTER(_I64), _P, _P, _P, _P])
    f["bh_load_csv"] = (C.c_int, [_P, C.c_char_p, _I64, C.POINTER(_I64)])
    for name, (res, args) in f.items():
        if hasattr(lib, name):
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
    return lib


def library():
    """The loaded libbh_gpu.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build the CUDA extension first "
                               "(python barnes-hut_gb300/build.py)")
        _lib = _sig(C.CDLL(str(LIB_PATH)))
    return _lib


def _check(rc: int) -> None:
    if rc != 0:
        raise BhError(rc, library().bh_last_error().decode(errors="replace"))


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f64(a, shape=None) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


def _u64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint64)


# ---------------------------------------------------------------- host side
def kepler_to_cartesian(elements) -> np.ndarray:
    """convertKeplerToCartesian for rows {e, a, i, omega, Omega, M, epoch, mu}."""
    el = _f64(elements).reshape(-1, 8)
    out = np.empty((el.shape[0], 6))
    _check(library().bh_kepler_to_cartesian(_ptr(el), el.shape[0], _ptr(out)))
    return out


def kepler_to_cartesian_gpu(elements) -> np.ndarray:
    """The same conversion, batched on the GPU (agrees to rounding)."""
    el = _f64(elements).reshape(-1, 8)
    out = np.empty((el.shape[0], 6))
    _check(library().bh_kepler_to_cartesian_gpu(_ptr(el), el.shape[0], _ptr(out)))
    return out


def generate_system(seed: int, n: int, frac_outer: float = 0.1, frac_trojan: float = 0.0):
    """Seeded synthetic solar system: (pos, vel, mass, ids)."""
    pos = np.empty((n, 3)); vel = np.empty((n, 3)); mass = np.empty(n); ids = np.empty(n, np.uint64)
    _check(library().bh_generate_system(seed, n, frac_outer, frac_trojan, _ptr(pos), _ptr(vel), _ptr(mass),
                                        _ptr(ids)))
    return pos, vel, mass, ids


def selftest(which: int, n: int, seed: int = 1) -> int:
    """Mismatches of a hot-path arithmetic helper against IEEE (bh_selftest)."""
    f = _I64(0)
    _check(library().bh_selftest(int(which), int(n), int(seed), C.byref(f)))
    return f.value


def _line_bound(path, body_count: int) -> int:
    """An upper bound on a CSV file's data rows: its newline count plus one
    (fewer with a body_count limit)."""
    lines = 1
    with open(path, "rb") as fh:
        while True:
            chunk = fh.read(16 << 20)
            if not chunk:
                break
            lines += chunk.count(b"\n")
    return min(lines, body_count) if body_count > 0 else lines


def _read_csv_with(fn, path, body_count: int):
    """One call of a reader entry point into arrays sized by the file's line
    count, so each skipped row's warning is printed once, as readCSV prints
    it."""
    p = str(path).encode()
    try:
        cap = _line_bound(path, body_count)
    except OSError:
        cap = 0  # the entry point reports the missing file
    ids = np.empty(cap, np.uint64); mass = np.empty(cap); pos = np.empty((max(cap, 1), 3))
    vel = np.empty((max(cap, 1), 3))
    n = _I64(0)
    _check(fn(p, body_count, C.byref(n), _ptr(ids), _ptr(mass), _ptr(pos), _ptr(vel)))
    k = n.value
    return ids[:k].copy(), mass[:k].copy(), pos[:k].copy(), vel[:k].copy()


def read_csv(path, body_count: int = -1):
    """readCSV: (ids, mass, pos, vel)."""
    return _read_csv_with(library().bh_read_csv, path, body_count)


def read_csv_gpu(path, body_count: int = -1):
    """readCSV parsed on the GPU: (ids, mass, pos, vel), as read_csv."""
    return _read_csv_with(library().bh_read_csv_gpu, path, body_count)


def write_csv(path, ids, mass, pos, vel) -> None:
    ids = _u64(ids); mass = _f64(mass); pos = _f64(pos); vel = _f64(vel)
    _check(library().bh_write_csv(str(path).encode(), len(mass), _ptr(ids), _ptr(mass), _ptr(pos), _ptr(vel)))


def write_vtp(path, ids, mass, pos, vel, acc, rank: int = 0) -> None:
    """writeSnapshot: one VTK XML PolyData snapshot (ParaView)."""
    ids = _u64(ids); mass = _f64(mass); pos = _f64(pos); vel = _f64(vel); acc = _f64(acc)
    _check(library().bh_write_vtp(str(path).encode(), int(rank), len(mass), _ptr(ids), _ptr(mass), _ptr(pos),
                                  _ptr(vel), _ptr(acc)))


def let_bucket_boxes(prefixes, bucket_bits: int, bbox) -> np.ndarray:
    """The bucket boxes of a remote domain (exchangeEssentialTrees): one
    (6,) box per bucket prefix, {min.xyz, max.xyz}."""
    p = _u64(prefixes)
    out = np.empty((len(p), 6))
    _check(library().bh_let_bucket_boxes(_ptr(p), len(p), int(bucket_bits), _ptr(_f64(bbox)), _ptr(out)))
    return out


# ---------------------------------------------------------------- device context
class Context:
    """A device-resident body set on one GPU (bh_context)."""

    def __init__(self, capacity: int, device: int = 0):
        self._h = C.c_void_p()
        _check(library().bh_context_create(int(capacity), int(device), C.byref(self._h)))
        self.capacity = int(capacity)

    def close(self) -> None:
        if self._h:
            library().bh_context_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    @property
    def n(self) -> int:
        v = _I64(0)
        _check(library().bh_num_bodies(self._h, C.byref(v)))
        return v.value

    def stream(self) -> int:
        s = C.c_void_p()
        _check(library().bh_context_stream(self._h, C.byref(s)))
        return s.value or 0

    def sync(self) -> None:
        _check(library().bh_context_sync(self._h))

    def set_bodies(self, pos, vel, mass, ids=None) -> None:
        pos = _f64(pos).reshape(-1, 3)
        n = pos.shape[0]
        vel = _f64(vel).reshape(n, 3)
        mass = _f64(mass).reshape(n)
        ids = np.arange(n, dtype=np.uint64) if ids is None else _u64(ids)
        _check(library().bh_set_bodies(self._h, n, _ptr(pos), _ptr(vel), _ptr(mass), _ptr(ids)))

    def load_csv(self, path, body_count: int = -1) -> int:
        """readCSV parsed on the GPU into this context's bodies; returns n."""
        n = _I64(0)
        _check(library().bh_load_csv(self._h, str(path).encode(), body_count, C.byref(n)))
        return n.value

    def set_accelerations(self, acc) -> None:
        acc = _f64(acc).reshape(-1, 3)
        _check(library().bh_set_accelerations(self._h, _ptr(acc)))

    def get_bodies(self, out=None):
        """(pos, vel, mass, ids, acc) in the current (last sorted) order;
        `out` may supply the five destination arrays (e.g. pinned memory)."""
        n = self.n
        if out is None:
            out = (np.empty((n, 3)), np.empty((n, 3)), np.empty(n), np.empty(n, np.uint64), np.empty((n, 3)))
        pos, vel, mass, ids, acc = out
        _check(library().bh_get_bodies(self._h, _ptr(pos), _ptr(vel), _ptr(mass), _ptr(ids), _ptr(acc)))
        return pos, vel, mass, ids, acc

    def compute_bbox(self) -> np.ndarray:
        out = np.empty(6)
        _check(library().bh_compute_bbox(self._h, _ptr(out)))
        return out

    def set_bbox(self, bbox) -> None:
        """The global box (e.g. over all ranks' bodies) in place of
        compute_bbox."""
        _check(library().bh_set_bbox(self._h, _ptr(_f64(bbox))))

    def compute_keys(self) -> np.ndarray:
        out = np.empty(self.n, np.uint64)
        _check(library().bh_compute_keys(self._h, _ptr(out)))
        return out

    def sort_bodies(self) -> np.ndarray:
        perm = np.empty(self.n, np.int64)
        _check(library().bh_sort_bodies(self._h, _ptr(perm)))
        return perm

    def build_tree(self, merge: bool = True) -> None:
        """buildOctreeBottomUp, with (default) or without the single-rank
        exchange merge."""
        if merge:
            _check(library().bh_build_tree(self._h))
        else:
            _check(library().bh_build_tree_options(self._h, 0))

    def tree_info(self):
        r, nn, nl = _I64(0), _I64(0), _I64(0)
        _check(library().bh_tree_info(self._h, C.byref(r), C.byref(nn), C.byref(nl)))
        return {"records": r.value, "nodes": nn.value, "leaves": nl.value}

    def _tree_nodes(self) -> int:
        """The device node count (counts only, no copy of the tree)."""
        nn = _I64(0)
        _check(library().bh_tree_info(self._h, None, C.byref(nn), None))
        return nn.value

    def tree_slots(self):
        """(prefix u64, depth u8) of the reference cell each device node
        stands for (the deepest cell of its single-child chain)."""
        k = self._tree_nodes()
        p = np.empty(k, np.uint64); d = np.empty(k, np.uint8)
        _check(library().bh_tree_slots(self._h, _ptr(p), _ptr(d)))
        return p, d

    def tree_spread(self) -> np.ndarray:
        """sqrt(Q/m) of the far-field masses per node (bh_tree_slots order)."""
        out = np.empty(self._tree_nodes(), np.float32)
        _check(library().bh_tree_spread(self._h, _ptr(out)))
        return out

    def export_tree(self):
        """The reference's node set sorted by (depth, prefix):
        (prefix u64, depth u8, mass f64, com (k,3) f64)."""
        k = self.tree_info()["records"]
        prefix = np.empty(k, np.uint64); depth = np.empty(k, np.uint8); mass = np.empty(k)
        com = np.empty((k, 3))
        _check(library().bh_export_tree(self._h, _ptr(prefix), _ptr(depth), _ptr(mass), _ptr(com)))
        return prefix, depth, mass, com

    def let_export(self, boxes, bbox, theta2: float, max_depth: int = 21):
        """createInteractionListForRank on the tree in place: the cells a
        remote domain (boxes, (k, 6)) needs, as (prefix u64, depth u8,
        mass f64, com (k, 3) f64) in the tree's node order."""
        bx = _f64(boxes).reshape(-1, 6)
        cap = self._tree_nodes()
        prefix = np.empty(cap, np.uint64); depth = np.empty(cap, np.uint8); mass = np.empty(cap)
        com = np.empty((cap, 3))
        k = _I64(0)
        _check(library().bh_let_export(self._h, _ptr(bx), bx.shape[0], _ptr(_f64(bbox)), float(theta2),
                                       int(max_depth), cap, _ptr(prefix), _ptr(depth), _ptr(mass), _ptr(com),
                                       C.byref(k)))
        k = k.value
        return prefix[:k], depth[:k], mass[:k], com[:k]

    def pseudo_leaf_tree(self, prefix, depth, mass, com):
        """buildTreeFromPseudoLeaves over received records on this context's
        device: the map's cells sorted by (depth, prefix), as (prefix u64,
        depth u8, mass f64, com (k, 3) f64)."""
        p = _u64(prefix); d = np.ascontiguousarray(depth, np.uint8); m = _f64(mass)
        c = _f64(com).reshape(-1, 3)
        cap = int(np.sum(np.minimum(d.astype(np.int64), 21) + 1)) if len(d) else 0
        op = np.empty(cap, np.uint64); od = np.empty(cap, np.uint8); om = np.empty(cap); oc = np.empty((cap, 3))
        k = _I64(0)
        _check(library().bh_pseudo_leaf_tree(self._h, _ptr(p), _ptr(d), _ptr(m), _ptr(c), len(p), cap, _ptr(op),
                                             _ptr(od), _ptr(om), _ptr(oc), C.byref(k)))
        k = k.value
        return op[:k], od[:k], om[:k], oc[:k]

    def let_accelerations(self, prefix, depth, mass, com, theta=THETA_DEFAULT, G=G_DEFAULT, soft2=0.0,
                          direct=False) -> np.ndarray:
        """computeAccelerationsWithLET (direct=False) or
        computeAccelerationsWithRemoteDirectSum (direct=True) for the local
        bodies (current order) with the received records."""
        p = _u64(prefix); d = np.ascontiguousarray(depth, np.uint8); m = _f64(mass)
        c = _f64(com).reshape(-1, 3)
        out = np.empty((self.n, 3))
        fn = library().bh_let_direct_accelerations if direct else library().bh_let_accelerations
        _check(fn(self._h, _ptr(p), _ptr(d), _ptr(m), _ptr(c), len(m), float(theta), float(G), float(soft2),
                  _ptr(out)))
        return out

    def compute_accelerations(self, theta=THETA_DEFAULT, G=G_DEFAULT, soft2=0.0, mode=MODE_PLAIN_FP64,
                              download=True):
        out = np.empty((self.n, 3)) if download else None
        _check(library().bh_compute_accelerations(self._h, theta, G, soft2, mode, _ptr(out)))
        return out

    def interaction_counts(self) -> np.ndarray:
        """Accepted interactions per body of the last force evaluation."""
        out = np.empty(self.n, np.int32)
        _check(library().bh_interaction_counts(self._h, _ptr(out)))
        return out

    def interaction_count(self) -> int:
        v = _I64(0)
        _check(library().bh_interaction_count(self._h, C.byref(v)))
        return v.value

    def set_step_graphs(self, on: bool) -> None:
        """Replay kicked steps through a captured CUDA graph (default on)."""
        _check(library().bh_set_step_graphs(self._h, 1 if on else 0))

    def set_profiling(self, on: bool = True) -> None:
        _check(library().bh_set_profiling(self._h, 1 if on else 0))

    PHASES = ("kick_drift_bbox", "keys", "sort", "permute", "build", "forces")

    def phase_times(self):
        """(dict phase -> accumulated device ms, kernel launches so far)."""
        ms = np.zeros(8)
        nl = _I64(0)
        _check(library().bh_phase_times(self._h, _ptr(ms), C.byref(nl)))
        return dict(zip(self.PHASES, ms[:6].tolist())), nl.value

    def launches(self) -> int:
        return self.phase_times()[1]

    def measure_fma_peak(self, fp64: bool = True) -> float:
        v = _D(0.0)
        _check(library().bh_measure_fma_peak(self._h, 1 if fp64 else 0, C.byref(v)))
        return v.value

    def direct_sum(self, targets, G=G_DEFAULT) -> np.ndarray:
        """FP64 direct-sum accelerations of the bodies at positions `targets`
        of the current order."""
        t = np.ascontiguousarray(targets, np.int64)
        out = np.empty((len(t), 3))
        _check(library().bh_direct_sum(self._h, len(t), _ptr(t), G, _ptr(out)))
        return out

    def invariants(self, G=G_DEFAULT, theta=THETA_DEFAULT) -> dict:
        """E, K, U, L (3), P (3).  theta = 0: exact pair potential (N <= 131072);
        theta > 0: massive-body pairs exact, the rest through the tree."""
        out = np.empty(9)
        _check(library().bh_invariants(self._h, G, theta, _ptr(out)))
        return dict(E=out[0], K=out[1], U=out[2], L=out[3:6].copy(), P=out[6:9].copy())

    def learned_collect(self, theta=THETA_DEFAULT, theta_label=0.5, theta_max=3.0, G=G_DEFAULT,
                        max_pairs=2_000_000):
        """(features (k, 8), labels (k,)) training pairs from the current tree."""
        F = np.empty((max_pairs, 8), np.float32); L = np.empty(max_pairs, np.float32)
        k = _I64(0)
        _check(library().bh_learned_collect(self._h, theta, theta_label, theta_max, G, max_pairs, _ptr(F), _ptr(L),
                                            C.byref(k)))
        return F[:k.value].copy(), L[:k.value].copy()

    def learned_set_model(self, params, scale, budget=1e-5, theta_max=3.0) -> None:
        p = np.ascontiguousarray(params, np.float32); sc = np.ascontiguousarray(scale, np.float32)
        _check(library().bh_learned_set_model(self._h, _ptr(p), _ptr(sc), budget, theta_max))

    def learned_set_criterion(self, band: float = 0.5, frac: float = 0.25) -> None:
        """Decades around the allowance the network decides; largest share of
        the remaining allowance one candidate takes."""
        _check(library().bh_learned_set_criterion(self._h, band, frac))

    def learned_stats(self) -> dict:
        v = np.zeros(4, np.int64)
        _check(library().bh_learned_stats(self._h, _ptr(v)))
        return {"candidates": int(v[0]), "accepted": int(v[1]), "fallback": int(v[2]), "analytic": int(v[3])}

    def step(self, dt, theta=THETA_DEFAULT, G=G_DEFAULT, nsteps=1, mode=MODE_PLAIN_FP64, t=None) -> float:
        tv = _D(0.0 if t is None else t)
        _check(library().bh_step(self._h, dt, theta, G, int(nsteps), mode, None if t is None else C.byref(tv)))
        return tv.value

    def step_host(self, pos, vel, mass, ids, acc, dt, theta=THETA_DEFAULT, G=G_DEFAULT, nsteps=1,
                  mode=MODE_PLAIN_FP64, t=0.0) -> float:
        """bh_step_host: `nsteps` steps of a host-resident state, updated in
        place (pos, vel: (n, 3) float64; mass; ids uint64; acc (n, 3), the
        previous step's accelerations in, the last step's out), in one call
        with one synchronisation.  Returns the new time."""
        arrays = (pos, vel, mass, ids, acc)
        for a in arrays:
            if not (isinstance(a, np.ndarray) and a.flags.c_contiguous and a.flags.writeable):
                raise ValueError("step_host: arrays must be writeable C-contiguous numpy arrays")
        n = len(mass)
        if pos.shape != (n, 3) or vel.shape != (n, 3) or acc.shape != (n, 3) or ids.shape != (n,) or \
                pos.dtype != np.float64 or vel.dtype != np.float64 or acc.dtype != np.float64 or \
                mass.dtype != np.float64 or ids.dtype != np.uint64:
            raise ValueError("step_host: expected (n, 3) float64 pos/vel/acc, float64 mass, uint64 ids")
        tv = _D(t)
        _check(library().bh_step_host(self._h, n, _ptr(pos), _ptr(vel), _ptr(mass), _ptr(ids), _ptr(acc), dt,
                                      theta, G, int(nsteps), mode, C.byref(tv)))
        return tv.value


# ------------------------------------------------- learned acceptance network
MLP_PARAMS = 4801
MLP_SCALE = 34


def mlp_gradient(params, X, T):
    """(loss, gradient) of the network on standardised X (n, 8), targets T."""
    p = np.ascontiguousarray(params, np.float32)
    X = np.ascontiguousarray(X, np.float32).reshape(-1, 8)
    T = np.ascontiguousarray(T, np.float32)
    g = np.empty(MLP_PARAMS, np.float32)
    loss = C.c_float(0.0)
    _check(library().bh_mlp_gradient(_ptr(p), _ptr(X), _ptr(T), len(T), _ptr(g), C.byref(loss)))
    return loss.value, g


def mlp_train(features, labels, epochs=20, batch=4096, lr=2e-3, seed=0):
    """Trains the acceptance network on the GPU: (params, scale, losses)."""
    F = np.ascontiguousarray(features, np.float32).reshape(-1, 8)
    L = np.ascontiguousarray(labels, np.float32)
    params = np.empty(MLP_PARAMS, np.float32)
    scale = np.empty(MLP_SCALE, np.float32)
    losses = np.empty(epochs, np.float32)
    _check(library().bh_mlp_train(_ptr(F), _ptr(L), len(L), epochs, batch, lr, seed, _ptr(params), _ptr(scale),
                                  _ptr(losses)))
    return params, scale, losses


def mlp_save(path, params, scale) -> None:
    """Writes a trained model (parameters and feature scaling) to a file."""
    p = np.ascontiguousarray(params, np.float32); sc = np.ascontiguousarray(scale, np.float32)
    if p.size != MLP_PARAMS or sc.size != MLP_SCALE:
        raise ValueError("mlp_save: wrong parameter or scale count")
    _check(library().bh_mlp_save(str(path).encode(), _ptr(p), _ptr(sc)))


def mlp_load(path):
    """(params, scale) of a model file written by mlp_save / bh_mlp_save."""
    p = np.empty(MLP_PARAMS, np.float32); sc = np.empty(MLP_SCALE, np.float32)
    _check(library().bh_mlp_load(str(path).encode(), _ptr(p), _ptr(sc)))
    return p, sc


def mlp_predict(params, scale, features):
    """Predicted log10 error of raw feature rows (fused inference path) and
    the in-training-range flags."""
    p = np.ascontiguousarray(params, np.float32); sc = np.ascontiguousarray(scale, np.float32)
    F = np.ascontiguousarray(features, np.float32).reshape(-1, 8)
    out = np.empty(len(F), np.float32); inr = np.empty(len(F), np.int32)
    _check(library().bh_mlp_predict(_ptr(p), _ptr(sc), _ptr(F), len(F), _ptr(out), _ptr(inr)))
    return out, inr.astype(bool)


# ------------------------------------------------- reference-named functions
def compute_local_bbox(pos) -> np.ndarray:
    pos = _f64(pos).reshape(-1, 3)
    out = np.empty(6)
    _check(library().bh_compute_local_bbox(_ptr(pos), pos.shape[0], _ptr(out)))
    return out


def generateMortonCodes(pos, bbox) -> np.ndarray:  # noqa: N802 (reference name)
    pos = _f64(pos).reshape(-1, 3)
    bb = _f64(bbox).reshape(6)
    out = np.empty(pos.shape[0], np.uint64)
    _check(library().bh_generate_morton_codes(_ptr(pos), pos.shape[0], _ptr(bb), _ptr(out)))
    return out


def sortBodiesByMortonKey(keys, pos, mass, vel, ids):  # noqa: N802
    """Returns sorted copies (keys, pos, mass, vel, ids)."""
    keys = _u64(keys).copy(); pos = _f64(pos).reshape(-1, 3).copy(); mass = _f64(mass).copy()
    vel = _f64(vel).reshape(-1, 3).copy(); ids = _u64(ids).copy()
    _check(library().bh_sort_bodies_by_morton_key(len(keys), _ptr(keys), _ptr(pos), _ptr(mass), _ptr(vel),
                                                  _ptr(ids)))
    return keys, pos, mass, vel, ids


def buildOctreeBottomUp(pos, vel, mass, ids=None, ctx: Context | None = None):  # noqa: N802
    """Loads the bodies, computes bbox/keys, sorts and builds; returns the
    context holding the tree (export with ``ctx.export_tree()``)."""
    pos = _f64(pos).reshape(-1, 3)
    own = ctx is None
    if own:
        ctx = Context(max(1, pos.shape[0]))
    ctx.set_bodies(pos, vel, mass, ids)
    ctx.compute_bbox()
    ctx.compute_keys()
    ctx.sort_bodies()
    ctx.build_tree()
    return ctx


def computeAccelerations(ctx: Context, theta=THETA_DEFAULT, G=G_DEFAULT, soft2=0.0,  # noqa: N802
                         mode=MODE_PLAIN_FP64) -> np.ndarray:
    return ctx.compute_accelerations(theta, G, soft2, mode)
