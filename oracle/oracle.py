"""ctypes access to the CPU oracle (TEST INFRASTRUCTURE ONLY).

Two libraries can sit behind this module:

* ``oracle/_build/libcp3oracle.so`` -- the C restatement in ``cp3_oracle.c`` (built on any
  machine by ``make -C oracle``); ``libcp3oracle_fast.so`` is the same source built with the
  compiler's default FMA contraction and is what bench.py times as the CPU baseline.
* ``oracle/_ref/libcp3ref.so`` -- the reference's own CPU propagators compiled from the
  reference tree (``make -C oracle ref REF=<tree>``); only present where the reference
  sources are.  ``libcp3ref_fast.so`` is the same with the compiler's default contraction
  (the timed reference arm), and ``refgpu_bench`` runs the reference's own FP64 CUDA
  propagators (``make -C oracle refgpu``).  ``reference_dir()`` says where the tree is.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REFDIR = os.path.join(HERE, "_ref")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class _Mixing(C.Structure):
    _fields_ = [("theta12", C.c_double), ("theta13", C.c_double), ("theta23", C.c_double),
                ("dcp", C.c_double), ("knutype", C.c_int), ("dm12sq", C.c_double),
                ("dm23sq", C.c_double)]


class _Earth(C.Structure):
    _fields_ = [("n", C.c_int), ("radii", _dp), ("rhos", _dp), ("yps", _dp), ("as_", _dp),
                ("bs", _dp), ("cs", _dp), ("poly", C.c_int)]


@dataclass
class Mixing:
    """Oscillation parameters as handed to setMNSMatrix / setNeutrinoMasses."""
    theta12: float
    theta13: float
    theta23: float
    dcp: float
    dm12sq: float
    dm23sq: float
    knutype: int = 1

    def c(self) -> _Mixing:
        return _Mixing(self.theta12, self.theta13, self.theta23, self.dcp, self.knutype,
                       self.dm12sq, self.dm23sq)


def _ptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(_dp)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def build(quiet: bool = True) -> None:
    """Compile the C restatement (both variants) with the committed Makefile, or with the
    same gcc commands directly where make is absent."""
    try:
        out = subprocess.run(["make", "-s", "-C", HERE, "all"], capture_output=True, text=True)
        if out.returncode == 0:
            return
        msg = out.stdout + out.stderr
    except FileNotFoundError:
        msg = "make not found"
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "cp3_oracle.c")
    base = ["gcc", "-std=c11", "-D_DEFAULT_SOURCE", "-O3", "-fopenmp", "-fPIC", "-shared"]
    for extra, name in ((["-ffp-contract=off"], "libcp3oracle.so"), ([], "libcp3oracle_fast.so")):
        r = subprocess.run(base + extra + ["-o", os.path.join(BUILD, name), src, "-lm"],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + msg + "\n" + r.stdout + r.stderr)


class OracleError(RuntimeError):
    pass


def reference_dir():
    """The reference source tree, or None: $CP3_REFERENCE_DIR if set, else the untracked copy
    at <repo>/baseline/_ref (git-ignored; it travels with the working tree to a GPU host)."""
    for cand in (os.environ.get("CP3_REFERENCE_DIR"),
                 os.path.join(os.path.dirname(HERE), "baseline", "_ref")):
        if cand and os.path.isfile(os.path.join(cand, "physics.hpp")):
            return os.path.abspath(cand)
    return None


def build_reference(gpu: bool = True) -> dict:
    """Compile the reference's CPU propagators (and, with ``gpu``, its CUDA timing driver)
    from reference_dir() into oracle/_ref.  Returns {target: ok} ({} without a tree)."""
    ref = reference_dir()
    if ref is None:
        return {}
    done = {}
    for target in (["ref", "refgpu"] if gpu else ["ref"]):
        r = subprocess.run(["make", "-s", "-j3", "-C", HERE, target, f"REF={ref}"],
                           capture_output=True, text=True)
        done[target] = r.returncode == 0
        if r.returncode != 0:
            with open(os.path.join(REFDIR if os.path.isdir(REFDIR) else HERE,
                                   f"build_{target}.log"), "w") as f:
                f.write(r.stdout + r.stderr)
    return done


_ORC_MSG = {1: "bad size", 2: "radii order messed up", 3: "invalid number of maxLayer",
            4: "bad argument"}


class Oracle:
    """The C restatement. ``fast=True`` loads the contraction-enabled build (timing only)."""

    def __init__(self, fast: bool = False):
        name = "libcp3oracle_fast.so" if fast else "libcp3oracle.so"
        path = os.path.join(BUILD, name)
        if not os.path.exists(path):
            build()
        lib = C.CDLL(path)
        lib.orc_atmos.argtypes = [C.POINTER(_Mixing), C.c_int, _dp, C.c_int, _dp, C.c_int,
                                  C.POINTER(_Earth), C.c_double, C.c_int, C.c_int, _dp, _dp,
                                  C.c_int, C.c_int, _dp]
        lib.orc_beam.argtypes = [C.POINTER(_Mixing), C.c_int, _dp, C.c_int, C.c_double,
                                 C.c_double, C.c_int, _dp]
        lib.orc_max_layers.argtypes = [_dp, C.c_int, _dp, C.c_int, C.c_int, _ip]
        lib.orc_flip_model.argtypes = [C.c_int] + [_dp] * 10
        lib.orc_trajectory.argtypes = [C.POINTER(_Earth), C.c_double, C.c_double, C.c_int, _dp,
                                       _dp]
        lib.orc_transition_matrix.argtypes = [C.POINTER(_Mixing), C.c_int, C.c_double,
                                              C.c_double, C.c_double, _dp]
        self.lib = lib

    # -- model handling (AtmosCpuPropagator::setDensity) -------------------------------
    def flip_model(self, radii, *cols):
        radii = _f64(radii)
        n = len(radii)
        cols = [_f64(c) for c in cols] + [None] * (4 - len(cols))
        outs = [np.empty(n) if c is not None else None for c in cols]
        r_out = np.empty(n)
        rc = self.lib.orc_flip_model(n, _ptr(radii), *[_ptr(c) for c in cols], _ptr(r_out),
                                     *[_ptr(o) for o in outs])
        if rc:
            raise OracleError(_ORC_MSG.get(rc, str(rc)))
        return (r_out,) + tuple(o for o in outs if o is not None)

    def _earth(self, radii, rhos, yps, poly_abc=None):
        """Flip to descending order and pack. Keeps the arrays alive on the struct."""
        if poly_abc is not None:
            r, a, b, c, y = self.flip_model(radii, poly_abc[0], poly_abc[1], poly_abc[2], yps)
            e = _Earth(len(r), _ptr(r), None, _ptr(y), _ptr(a), _ptr(b), _ptr(c), 1)
            e._keep = (r, a, b, c, y)
        else:
            r, rho, y = self.flip_model(radii, rhos, yps)
            e = _Earth(len(r), _ptr(r), _ptr(rho), _ptr(y), None, None, None, 0)
            e._keep = (r, rho, y)
        return e

    def max_layers(self, radii_desc, cosines, limit=64):
        r = _f64(radii_desc)
        cz = _f64(cosines)
        out = np.empty(len(cz), dtype=np.int32)
        rc = self.lib.orc_max_layers(_ptr(r), len(r), _ptr(cz), len(cz), limit,
                                     out.ctypes.data_as(_ip))
        return out, rc

    def trajectory(self, radii, rhos, yps, cosine, h_km, poly_abc=None, limit=64):
        e = self._earth(radii, rhos, yps, poly_abc)
        m, _ = self.max_layers(e._keep[0], [cosine], limit)
        M = int(m[0])
        L = np.empty(M + 1)
        rho = np.empty(M + 1)
        self.lib.orc_trajectory(C.byref(e), float(cosine), float(h_km), M, _ptr(L), _ptr(rho))
        return L, rho

    # -- propagation --------------------------------------------------------------------
    def atmos(self, mix: Mixing, antineutrino: bool, cosines, energies, radii, rhos, yps,
              h_km: float, poly_abc=None, avg=None, layer_limit: int = 64,
              nthreads: int = 0) -> np.ndarray:
        """Probabilities [nc][ne][9] (channel a*3+b = P(a->b)), reference CPU layout."""
        cz = _f64(cosines)
        en = _f64(energies)
        e = self._earth(radii, rhos, yps, poly_abc)
        out = np.empty((len(cz), len(en), 9))
        nb, pp, pe = 0, None, None
        if avg is not None:
            nb = int(avg[0])
            pp = _f64(avg[1])
            pe = _f64(avg[2])
        rc = self.lib.orc_atmos(C.byref(mix.c()), int(bool(antineutrino)), _ptr(cz), len(cz),
                                _ptr(en), len(en), C.byref(e), float(h_km), int(nb > 0), nb,
                                _ptr(pp), _ptr(pe), layer_limit, nthreads, _ptr(out))
        if rc:
            raise OracleError(_ORC_MSG.get(rc, str(rc)))
        return out

    def beam(self, mix: Mixing, antineutrino: bool, energies, rho: float, L_km: float,
             nthreads: int = 0) -> np.ndarray:
        en = _f64(energies)
        out = np.empty((len(en), 9))
        rc = self.lib.orc_beam(C.byref(mix.c()), int(bool(antineutrino)), _ptr(en), len(en),
                               float(rho), float(L_km), nthreads, _ptr(out))
        if rc:
            raise OracleError(_ORC_MSG.get(rc, str(rc)))
        return out

    def transition_matrix(self, mix: Mixing, antineutrino: bool, E, rho_e, L_km):
        out = np.empty(18)
        self.lib.orc_transition_matrix(C.byref(mix.c()), int(bool(antineutrino)), float(E),
                                       float(rho_e), float(L_km), _ptr(out))
        return (out[0::2] + 1j * out[1::2]).reshape(3, 3)


class Reference:
    """The reference's own CPU propagators (only where oracle/_ref was built).  ``fast=True``
    loads the build with the compiler's default contraction, the one the reference arm times."""

    PATH = os.path.join(REFDIR, "libcp3ref.so")
    FAST_PATH = os.path.join(REFDIR, "libcp3ref_fast.so")
    GPU_BENCH = os.path.join(REFDIR, "refgpu_bench")

    @classmethod
    def available(cls, fast: bool = False) -> bool:
        return os.path.exists(cls.FAST_PATH if fast else cls.PATH)

    def __init__(self, fast: bool = False):
        lib = C.CDLL(self.FAST_PATH if fast else self.PATH)
        lib.ref_atmos.argtypes = ([C.c_double] * 4 + [C.c_int] + [C.c_double] * 2 + [C.c_int]
                                  + [_dp, C.c_int, _dp, C.c_int] + [_dp] * 5
                                  + [C.c_int, C.c_int, C.c_double, C.c_int, _dp, _dp, C.c_int,
                                     C.c_int, _dp, _dp])
        lib.ref_beam.argtypes = ([C.c_double] * 4 + [C.c_int] + [C.c_double] * 2 + [C.c_int]
                                 + [_dp, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int, _dp,
                                    _dp])
        lib.ref_last_error.restype = C.c_char_p
        self.lib = lib

    def atmos(self, mix: Mixing, antineutrino, cosines, energies, radii, rhos, yps, h_km,
              poly_abc=None, avg=None, nthreads=1, reps=0):
        cz, en, r, y = _f64(cosines), _f64(energies), _f64(radii), _f64(yps)
        if poly_abc is not None:
            c1, c2, c3 = (_f64(x) for x in poly_abc)
        else:
            c1, c2, c3 = _f64(rhos), None, None
        nb, pp, pe = 0, None, None
        if avg is not None:
            nb, pp, pe = int(avg[0]), _f64(avg[1]), _f64(avg[2])
        out = np.empty((len(cz), len(en), 9))
        secs = C.c_double(0.0)
        rc = self.lib.ref_atmos(mix.theta12, mix.theta13, mix.theta23, mix.dcp, mix.knutype,
                                mix.dm12sq, mix.dm23sq, int(bool(antineutrino)), _ptr(cz),
                                len(cz), _ptr(en), len(en), _ptr(r), _ptr(c1), _ptr(c2),
                                _ptr(c3), _ptr(y), len(r), int(poly_abc is not None),
                                float(h_km), nb, _ptr(pp), _ptr(pe), nthreads, reps,
                                C.cast(C.pointer(secs), _dp), _ptr(out))
        if rc:
            raise OracleError(self.lib.ref_last_error().decode())
        return (out, secs.value) if reps else out

    def beam(self, mix: Mixing, antineutrino, energies, rho, L_km, nthreads=1, reps=0):
        en = _f64(energies)
        out = np.empty((len(en), 9))
        secs = C.c_double(0.0)
        rc = self.lib.ref_beam(mix.theta12, mix.theta13, mix.theta23, mix.dcp, mix.knutype,
                               mix.dm12sq, mix.dm23sq, int(bool(antineutrino)), _ptr(en),
                               len(en), float(rho), float(L_km), nthreads, reps,
                               C.cast(C.pointer(secs), _dp), _ptr(out))
        if rc:
            raise OracleError(self.lib.ref_last_error().decode())
        return (out, secs.value) if reps else out
