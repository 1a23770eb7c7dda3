"""The reference's propagator classes over the C ABI.

Same class names, method names, argument meaning and error behaviour as CUDAProb3++'s
``AtmosCudaPropagatorSingle`` / ``BeamCudaPropagatorSingle`` (both ``Propagator<double>``),
so code and tests written against the reference read the same here.  Invalid input raises
``RuntimeError`` (the reference's ``std::runtime_error``) with the reference's message.

One addition: ``precision="mixed"`` selects the mixed-precision kernels (FP32 matrix work,
FP64 eigen-decomposition, double-float phases); the default ``"fp64"`` is the drop-in.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._abi import CP3Error, check
from .types import NeutrinoType, ProbType

_PRECISION = {"fp64": _abi.FP64, "double": _abi.FP64, "mixed": _abi.MIXED, "float": _abi.MIXED}


def _f64(x):
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
    return a, a.ctypes.data_as(C.POINTER(C.c_double))


class Propagator:
    """Propagator<FLOAT_T> (propagator.hpp:45-300): the setters every propagator shares."""

    def __init__(self, handle: C.c_void_p, precision: int):
        self._h = handle
        self._lib = _abi.lib()
        self.precision = precision

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.cp3_destroy(h)
            self._h = None

    def close(self):
        self.__del__()

    def _check(self, rc):
        check(rc, self._h)

    # -- Propagator ------------------------------------------------------------------------
    def setMNSMatrix(self, theta12, theta13, theta23, dCP, kNuType=1):
        """Angles in radians; kNuType < 0 flips the sign of dCP (propagator.hpp:148-183)."""
        self._check(self._lib.cp3_set_mns(self._h, float(theta12), float(theta13),
                                          float(theta23), float(dCP), int(kNuType)))

    def setNeutrinoMasses(self, dm12sq, dm23sq):
        """eV^2; dm23sq = m3^2 - m2^2 (propagator.hpp:188-209)."""
        self._check(self._lib.cp3_set_masses(self._h, float(dm12sq), float(dm23sq)))

    def setEnergyList(self, energies):
        a, p = _f64(energies)
        self._check(self._lib.cp3_set_energies(self._h, p, len(a)))

    def calculateProbabilities(self, type=NeutrinoType.Neutrino):
        self._check(self._lib.cp3_calculate(self._h, int(type)))

    # -- additions (no reference counterpart) -------------------------------------------------
    def calculate_async(self, type=NeutrinoType.Neutrino, stream=None):
        """Launch on a cudaStream_t (int handle, e.g. torch.cuda.current_stream().cuda_stream)."""
        self._check(self._lib.cp3_calculate_async(self._h, int(type),
                                                  C.c_void_p(stream) if stream else None))

    def calculate_to_host_async(self, type, dst_ptr: int, n_chunks: int = 0, stream=None):
        """Compute and copy the whole result (device layout) to page-locked host memory at
        dst_ptr, in n_chunks pipelined pieces (0: the library's default)."""
        self._check(self._lib.cp3_calculate_to_host_async(
            self._h, int(type), C.c_void_p(dst_ptr), int(n_chunks),
            C.c_void_p(stream) if stream else None))

    def synchronize(self):
        self._check(self._lib.cp3_synchronize(self._h))

    def device_result(self):
        """(device pointer, is_float, bytes) of the result in the device layout."""
        ptr, isf, nb = C.c_void_p(), C.c_int(), C.c_size_t()
        self._check(self._lib.cp3_device_result(self._h, C.byref(ptr), C.byref(isf), C.byref(nb)))
        return ptr.value, bool(isf.value), nb.value

    def set_profiling(self, enable: bool = True):
        self._check(self._lib.cp3_set_profiling(self._h, int(bool(enable))))

    def kernel_times(self):
        """(eigen-table ms, per-bin kernel ms) of the last compute (needs set_profiling)."""
        a, b = C.c_double(), C.c_double()
        self._check(self._lib.cp3_kernel_times(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def copy_result_async(self, dst_ptr: int, stream=None):
        self._check(self._lib.cp3_copy_result_async(self._h, C.c_void_p(dst_ptr),
                                                    C.c_void_p(stream) if stream else None))


class AtmosCudaPropagatorSingle(Propagator):
    """AtmosCudaPropagatorSingle (atmoscudapropagator.cuh:52-59):
    ``AtmosCudaPropagatorSingle(id, n_cosines, n_energies)`` or ``(n_cosines, n_energies)``."""

    def __init__(self, *args, precision: str = "fp64"):
        if len(args) == 2:
            dev, nc, ne = 0, args[0], args[1]
        elif len(args) == 3:
            dev, nc, ne = args
        else:
            raise TypeError("AtmosCudaPropagatorSingle(id, n_cosines, n_energies) or (n_cosines, n_energies)")
        L = _abi.lib()
        prec = _PRECISION[precision]
        h = C.c_void_p()
        rc = L.cp3_atmos_create(int(dev), int(nc), int(ne), prec, C.byref(h))
        if rc:
            raise CP3Error(rc, L.cp3_last_error(None).decode())
        super().__init__(h, prec)
        self.n_cosines, self.n_energies = int(nc), int(ne)
        self._avg_bins = 0

    def setCosineList(self, cosines):
        a, p = _f64(cosines)
        self._check(self._lib.cp3_set_cosines(self._h, p, len(a)))

    def setDensity(self, *args):
        """setDensity(radii, rhos, yps) | setDensity(radii, a, b, c, yps) | setDensity(rho)
        (atmoscpupropagator.hpp:116, 181, 347).  The one-argument form is the reference's
        printing dummy."""
        if len(args) == 1:
            print("DUMMY FUNCTION: ATMOS class uses setDensity(radii, rhos, yps), "
                  "setDensity(radii, a, b, c, yps) or setDensityFromFile(filename)")
            return
        if len(args) == 3:
            (r, pr), (rho, prho), (y, py) = (_f64(x) for x in args)
            if not (len(r) == len(rho)):
                raise RuntimeError("setDensity : rhos.size() != radii.size()")
            if not (len(rho) == len(y)):
                raise RuntimeError("setDensity : rhos.size() != yps.size()")
            if len(r) == 0:
                raise RuntimeError("setDensity : vectors must not be empty")
            self._check(self._lib.cp3_set_layers(self._h, pr, prho, py, len(r)))
            return
        if len(args) == 5:
            (r, pr), (a, pa), (b, pb), (c, pc), (y, py) = (_f64(x) for x in args)
            if len(a) != len(r):
                raise RuntimeError("setDensity : a.size() != radii.size()")
            if len(a) != len(y):
                raise RuntimeError("setDensity : a.size() != yps.size()")
            if min(len(a), len(b), len(c), len(r), len(y)) == 0:
                raise RuntimeError("setDensity : vectors must not be empty")
            self._check(self._lib.cp3_set_layers_poly(self._h, pr, pa, pb, pc, py, len(r)))
            return
        raise TypeError("setDensity takes 1, 3 or 5 arguments")

    def setDensityFromFile(self, filename, ye_core=0.468, ye_mantle=0.497):
        self._check(self._lib.cp3_set_density_file(self._h, str(filename).encode(),
                                                   float(ye_core), float(ye_mantle)))

    def setChemicalComposition(self, yps):
        a, p = _f64(yps)
        self._check(self._lib.cp3_set_chemical_composition(self._h, p, len(a)))

    def getNlayerBoundaries(self):
        """The density model's rows (layers + 1), as AtmosCpuPropagator::getNlayerBoundaries
        (atmoscpupropagator.hpp:85) after setDensityFromFile."""
        n = C.c_int()
        self._check(self._lib.cp3_get_n_layer_boundaries(self._h, C.byref(n)))
        return n.value

    def setProductionHeight(self, heightKM):
        self._check(self._lib.cp3_set_production_height(self._h, float(heightKM)))

    def setPathLength(self, path_length):
        print("DUMMY FUNCTION - ATMOS class calculates PATH LENGTH")

    def SetNumberOfProductionHeightBinsForAveraging(self, n_bins):
        """n_bins >= 1 enables averaging (the reference's switch never does; see
        atmoscpupropagator.hpp:97-99); setProductionHeightList must follow."""
        if n_bins > 20:
            raise RuntimeError("SetNumberOfProductionHeightBinsForAveraging : invalid number of "
                               "production height bins")
        self._avg_bins = int(n_bins)
        if n_bins == 0:
            self._check(self._lib.cp3_set_production_height_averaging(self._h, 0, None, None))

    def setProductionHeightList(self, list_prob, list_bins):
        if self._avg_bins < 1:
            raise RuntimeError("Propagator::setProductionHeightList. Trying to set Production "
                               "Height information but propagator is not expecting to use it")
        p, pp = _f64(list_prob)
        e, pe = _f64(list_bins)
        if len(p) != self._avg_bins * 2 * 3 * self.n_energies * self.n_cosines:
            raise RuntimeError("Propagator::setProductionHeightList. Prob array is not the expected size")
        if len(e) - 1 != self._avg_bins:
            raise RuntimeError("Propagator::setProductionHeightList. ProductionHeightBins array "
                               "is not expected size")
        self._check(self._lib.cp3_set_production_height_averaging(self._h, self._avg_bins, pp, pe))

    def getProbability(self, index_cosine, index_energy, t):
        out = C.c_double()
        self._check(self._lib.cp3_get_probability(self._h, int(index_cosine), int(index_energy),
                                                  int(t), C.byref(out)))
        return out.value

    def getProbabilityArr(self, t):
        """Energy-major, cosine-minor (atmoscudapropagator.cu:238-257)."""
        out = np.empty(self.n_cosines * self.n_energies)
        self._check(self._lib.cp3_get_probability_arr(self._h, int(t),
                                                      out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def result(self) -> np.ndarray:
        """Whole result [9][n_cosines][n_energies] (float64, or float32 for mixed)."""
        dt = np.float32 if self.precision == _abi.MIXED else np.float64
        out = np.empty((9, self.n_cosines, self.n_energies), dtype=dt)
        self.copy_result_async(out.ctypes.data)
        self.synchronize()
        return out

    def probabilities(self) -> np.ndarray:
        """Result as [n_cosines][n_energies][9] float64 (the reference CPU layout)."""
        return np.ascontiguousarray(np.transpose(self.result(), (1, 2, 0)), dtype=np.float64)


class BeamCudaPropagatorSingle(Propagator):
    """BeamCudaPropagatorSingle (beamcudapropagator.cuh:52-57):
    ``BeamCudaPropagatorSingle(id, n_energies, n_threads)`` or ``(n_energies, n_threads)``."""

    def __init__(self, *args, precision: str = "fp64"):
        if len(args) == 3:
            dev, ne = args[0], args[1]
        elif len(args) == 2:
            dev, ne = 0, args[0]
        elif len(args) == 1:
            dev, ne = 0, args[0]
        else:
            raise TypeError("BeamCudaPropagatorSingle(id, n_energies, n_threads) or (n_energies, n_threads)")
        L = _abi.lib()
        prec = _PRECISION[precision]
        h = C.c_void_p()
        rc = L.cp3_beam_create(int(dev), int(ne), prec, C.byref(h))
        if rc:
            raise CP3Error(rc, L.cp3_last_error(None).decode())
        super().__init__(h, prec)
        self.n_energies = int(ne)

    def setDensity(self, rho):
        self._check(self._lib.cp3_set_beam_density(self._h, float(rho)))

    def setPathLength(self, path_length):
        self._check(self._lib.cp3_set_beam_path_length(self._h, float(path_length)))

    def getProbability(self, index_energy, t):
        out = C.c_double()
        self._check(self._lib.cp3_get_probability_beam(self._h, int(index_energy), int(t),
                                                       C.byref(out)))
        return out.value

    def getProbabilityArr(self, t):
        out = np.empty(self.n_energies)
        self._check(self._lib.cp3_get_probability_arr(self._h, int(t),
                                                      out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def result(self) -> np.ndarray:
        dt = np.float32 if self.precision == _abi.MIXED else np.float64
        out = np.empty((9, self.n_energies), dtype=dt)
        self.copy_result_async(out.ctypes.data)
        self.synchronize()
        return out

    def probabilities(self) -> np.ndarray:
        """[n_energies][9] float64 (the reference CPU layout)."""
        return np.ascontiguousarray(self.result().T, dtype=np.float64)


def CudaPropagatorSingle(*args, float_type=np.float64):
    """The legacy template name CudaPropagatorSingle<FLOAT_T>(id, n_cosines, n_energies)
    (cudapropagator.cuh:40): FLOAT_T=double -> FP64 kernels, float -> mixed kernels."""
    prec = "fp64" if np.dtype(float_type) == np.float64 else "mixed"
    return AtmosCudaPropagatorSingle(*args, precision=prec)


__all__ = ["Propagator", "AtmosCudaPropagatorSingle", "BeamCudaPropagatorSingle",
           "CudaPropagatorSingle", "ProbType", "NeutrinoType"]
