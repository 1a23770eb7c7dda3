"""Batches: many propagation problems (parameter set x neutrino type x grid) computed by one
persistent, graph-captured launch (C ABI cp3_batch_*)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._abi import CP3Error
from .types import Mixing

_dp = C.POINTER(C.c_double)


def _f64(x):
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
    return a, a.ctypes.data_as(_dp)


class Batch:
    """Atmospheric and beam problems sharing one device, one persistent kernel per run."""

    def __init__(self, device: int = 0):
        self._lib = _abi.lib()
        h = C.c_void_p()
        rc = self._lib.cp3_batch_create(int(device), C.byref(h))
        if rc:
            raise CP3Error(rc, self._lib.cp3_batch_last_error(None).decode())
        self._h = h
        self.shapes = []  # (kind, rows, ne) per problem

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.cp3_batch_destroy(h)
            self._h = None

    def close(self):
        """Free the batch's device memory now (the handle is unusable afterwards)."""
        self.__del__()

    def _check(self, rc):
        if rc:
            raise CP3Error(rc, self._lib.cp3_batch_last_error(self._h).decode())

    def set_earth(self, radii, rho, ye, production_height_km):
        (r, pr), (d, pd), (y, py) = _f64(radii), _f64(rho), _f64(ye)
        self._check(self._lib.cp3_batch_set_earth(self._h, pr, pd, py, len(r),
                                                  float(production_height_km)))

    def add_atmos(self, cosines, energies) -> int:
        (c, pc), (e, pe) = _f64(cosines), _f64(energies)
        i = C.c_int()
        self._check(self._lib.cp3_batch_add_atmos(self._h, pc, len(c), pe, len(e), C.byref(i)))
        self.shapes.append(("atmos", len(c), len(e)))
        return i.value

    def add_beam(self, energies, rho, baselines_km) -> int:
        (e, pe), (L, pL) = _f64(energies), _f64(np.atleast_1d(baselines_km))
        i = C.c_int()
        self._check(self._lib.cp3_batch_add_beam(self._h, pe, len(e), float(rho), pL, len(L),
                                                 C.byref(i)))
        self.shapes.append(("beam", len(L), len(e)))
        return i.value

    def set_params(self, pid: int, m: Mixing, antineutrino: bool):
        knu = -1 if antineutrino else 1
        self._check(self._lib.cp3_batch_set_params(self._h, int(pid), m.theta12, m.theta13,
                                                   m.theta23, m.dcp, knu, m.dm12sq, m.dm23sq,
                                                   int(bool(antineutrino))))

    def commit(self):
        self._check(self._lib.cp3_batch_commit(self._h))

    def set_shape(self, rows_per_tile=1, blocks_per_sm=0, beam_chunk=4):
        self._check(self._lib.cp3_batch_set_shape(self._h, rows_per_tile, blocks_per_sm,
                                                  beam_chunk))

    def shape(self):
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        self._check(self._lib.cp3_batch_get_shape(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def set_split_tables(self, on: bool = True):
        """Tables and bins as two launches (True) or one launch with waits (False)."""
        self._check(self._lib.cp3_batch_set_split_tables(self._h, int(bool(on))))

    def split_tables(self) -> bool:
        v = C.c_int()
        self._check(self._lib.cp3_batch_get_split_tables(self._h, C.byref(v)))
        return bool(v.value)

    def debug_withhold_tables(self, on: bool = True):
        """Testing aid: runs hand out no eigen-table tile, so the bin tiles' bounded waits run
        out and synchronize() raises ("wait limit")."""
        self._check(self._lib.cp3_batch_debug_withhold_tables(self._h, int(bool(on))))

    def tune(self, use_cache=True):
        self._check(self._lib.cp3_batch_tune(self._h, int(bool(use_cache))))

    def run(self, stream=None):
        self._check(self._lib.cp3_batch_run(self._h, C.c_void_p(stream) if stream else None))

    def run_to_host(self, dst_ptr: int, n_pieces: int = 0, stream=None):
        """One run with every result copied to dst (result_bytes, laid out as the arena):
        the bins in windows of whole problems, each window's download overlapping the next
        window's computation.  Page-locked dst for the overlap."""
        self._check(self._lib.cp3_batch_run_to_host(self._h, C.c_void_p(dst_ptr), int(n_pieces),
                                                    C.c_void_p(stream) if stream else None))

    def synchronize(self) -> float:
        ms = C.c_double()
        self._check(self._lib.cp3_batch_synchronize(self._h, C.byref(ms)))
        return ms.value

    @staticmethod
    def parameter_bytes() -> int:
        """Bytes a run uploads per problem (its parameter block)."""
        return int(_abi.lib().cp3_batch_parameter_bytes())

    def info(self):
        n, bins, nbytes, tiles = C.c_int(), C.c_longlong(), C.c_size_t(), C.c_longlong()
        self._check(self._lib.cp3_batch_info(self._h, C.byref(n), C.byref(bins), C.byref(nbytes),
                                             C.byref(tiles)))
        return dict(problems=n.value, bins=bins.value, result_bytes=nbytes.value,
                    tiles=tiles.value)

    def result_ptr(self, pid: int):
        p, n = C.c_void_p(), C.c_size_t()
        self._check(self._lib.cp3_batch_result(self._h, int(pid), C.byref(p), C.byref(n)))
        return p.value, n.value

    def copy_result_async(self, pid: int, dst_ptr: int, stream=None):
        self._check(self._lib.cp3_batch_copy_result(self._h, int(pid), C.c_void_p(dst_ptr),
                                                    C.c_void_p(stream) if stream else None))

    def result_offset(self, pid: int) -> int:
        """Float offset of one problem's result in the batch's result arena."""
        off = C.c_size_t()
        self._check(self._lib.cp3_batch_result_offset(self._h, int(pid), C.byref(off)))
        return off.value

    def copy_results_async(self, first: int, count: int, dst_ptr: int, stream=None):
        """Asynchronous copy of the result arena's floats [first, first + count) to dst."""
        self._check(self._lib.cp3_batch_copy_results(self._h, int(first), int(count),
                                                     C.c_void_p(dst_ptr),
                                                     C.c_void_p(stream) if stream else None))

    def result(self, pid: int) -> np.ndarray:
        """Copy of one problem's result: atmospheric [9][nc][ne], beam [nL][9][ne]."""
        _, n = self.result_ptr(pid)
        kind, rows, ne = self.shapes[pid]
        out = np.empty(n, dtype=np.float32)
        self.synchronize()
        self.copy_result_async(pid, out.ctypes.data)
        self.synchronize_stream()
        return out.reshape((9, rows, ne) if kind == "atmos" else (rows, 9, ne))

    def synchronize_stream(self):
        """Waits for everything queued on the batch's own stream (result copies)."""
        self._check(self._lib.cp3_batch_synchronize(self._h, None))
