"""ORACLE -- test infrastructure only.

ctypes front end of oracle/neighbors.c, the CPU restatement of the
reference's radius graph (src/mlff_distiller/models/student_model.py:63-109)
plus the orthorhombic minimum-image rule used for periodic boxes (no
reference counterpart: the reference ignores pbc, student_model.py:694-703).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle_nbr.so")
_lib = None


def build() -> str:
    """Compile oracle/neighbors.c with the committed Makefile."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH) or (
            os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "neighbors.c"))
        ):
            build()
        lib = ctypes.CDLL(_LIB_PATH)
        i64p = ctypes.POINTER(ctypes.c_int64)
        lib.oracle_radius_graph.restype = ctypes.c_int64
        lib.oracle_radius_graph.argtypes = [
            ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_float,
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
        ]
        lib.oracle_radius_graph_pbc_cells.restype = ctypes.c_int64
        lib.oracle_radius_graph_pbc_cells.argtypes = [
            ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_float,
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
        ]
        lib.oracle_pair_distance.restype = ctypes.c_float
        lib.oracle_pair_distance.argtypes = [ctypes.c_float] * 3
        del i64p
        _lib = lib
    return _lib


def pair_distance(d: np.ndarray) -> np.ndarray:
    """float32 |d| by the reference's rounding recipe, one pair at a time."""
    lib = _load()
    d = np.asarray(d, dtype=np.float32).reshape(-1, 3)
    return np.array([lib.oracle_pair_distance(*map(float, r)) for r in d], dtype=np.float32)


def radius_graph(pos, mol_ptr, cutoff=5.0, box=None, pbc=None):
    """Edges (src, dst, shift) of every molecule, in the reference's order.

    pos: float32 [N,3]; mol_ptr: int64 [B+1] (molecule m owns atoms
    mol_ptr[m]..mol_ptr[m+1]-1); box: float32 [B,3] orthorhombic edge
    lengths; pbc: bool [B] (all three axes periodic or none).
    Returns src, dst (int64 [E]) and shift (int32 [E,3]) with
    r_e = pos[src] - pos[dst] + shift * box[mol].
    """
    lib = _load()
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    mol_ptr = np.ascontiguousarray(mol_ptr, dtype=np.int64)
    n_mol = len(mol_ptr) - 1
    if box is None:
        box = np.zeros((n_mol, 3), np.float32)
    box = np.ascontiguousarray(box, dtype=np.float32).reshape(n_mol, 3)
    if pbc is None:
        pbc = np.zeros(n_mol, np.uint8)
    pbc = np.ascontiguousarray(pbc, dtype=np.uint8).reshape(n_mol)
    n = pos.shape[0]
    # single large periodic box: cell-list candidates, same decision
    if n_mol == 1 and pbc[0] and n > 4000:
        cap = max(64 * n, 1024)
        while True:
            src = np.empty(cap, np.int64)
            dst = np.empty(cap, np.int64)
            sh = np.empty((cap, 3), np.int32)
            e = lib.oracle_radius_graph_pbc_cells(
                pos.ctypes.data, n, box.ctypes.data, float(cutoff),
                src.ctypes.data, dst.ctypes.data, sh.ctypes.data, cap)
            if e < 0:
                raise ValueError("periodic box edge shorter than 2*cutoff")
            if e <= cap:
                return src[:e], dst[:e], sh[:e]
            cap = int(e)
    cap = max(64 * n, 1024)
    while True:
        src = np.empty(cap, np.int64)
        dst = np.empty(cap, np.int64)
        sh = np.empty((cap, 3), np.int32)
        e = lib.oracle_radius_graph(
            pos.ctypes.data, n, mol_ptr.ctypes.data, n_mol,
            box.ctypes.data, pbc.ctypes.data, float(cutoff),
            src.ctypes.data, dst.ctypes.data, sh.ctypes.data, cap)
        if e < 0:
            raise ValueError("periodic box edge shorter than 2*cutoff")
        if e <= cap:
            return src[:e], dst[:e], sh[:e]
        cap = int(e)
