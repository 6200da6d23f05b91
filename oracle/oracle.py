"""ctypes wrapper of the FP64 CPU oracle (oracle/bear_oracle.c).

TEST INFRASTRUCTURE: only the tests, the smoke check and the benchmark's CPU
baseline leg use this module, and only as the checker / baseline. It builds
liboracle.so on first use if it is missing.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "bear_oracle.c")
LIB = os.path.join(HERE, "liboracle.so")

_dp = C.POINTER(C.c_double)
_lib = None


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
                               "-o", LIB, SRC, "-lm"])
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.c_char_p]
        L.orc_add_observation.restype = C.c_int
        L.orc_add_observation.argtypes = [C.c_void_p, C.c_char_p, C.c_char_p, C.c_int, _dp, _dp, _dp,
                                          _dp, _dp, C.c_int, _dp, _dp, C.c_char_p, C.c_char_p]
        L.orc_finalize.restype = C.c_int
        L.orc_finalize.argtypes = [C.c_void_p]
        for fn in ("orc_nb_spectral_points", "orc_nb_obs_points", "orc_nb_parameters"):
            getattr(L, fn).restype = C.c_int
            getattr(L, fn).argtypes = [C.c_void_p]
        L.orc_grid.argtypes = [C.c_void_p, _dp]
        L.orc_forward.restype = C.c_int
        L.orc_forward.argtypes = [C.c_void_p, _dp, C.c_int, _dp, _dp, C.POINTER(C.c_int)]
        L.orc_contribution.restype = C.c_int
        L.orc_contribution.argtypes = [C.c_void_p, _dp, C.c_int, _dp, _dp]
        L.orc_loglike.restype = C.c_int
        L.orc_loglike.argtypes = [C.c_void_p, _dp, C.c_int, _dp, _dp]
        L.orc_last_error.restype = C.c_char_p
        L.orc_set_threads.restype = C.c_int
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_set_tau_cutoff.restype = C.c_int
        L.orc_set_tau_cutoff.argtypes = [C.c_void_p, C.c_double]
        L.orc_obs_setup.restype = C.c_int
        L.orc_obs_setup.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_long), C.c_int]
        L.orc_destroy.restype = None
        L.orc_destroy.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def _ptr(a: Optional[np.ndarray]):
    if a is None:
        return C.cast(None, _dp)
    return a.ctypes.data_as(_dp)


class OracleModel:
    """A forward model + likelihood on the CPU, in FP64, built from the same
    config text and observation arrays the engine takes."""

    def __init__(self, config_text: str, observations: Sequence):
        L = lib()
        self._keep = []
        h = L.orc_create(config_text.encode())
        if not h:
            raise RuntimeError("oracle: " + L.orc_last_error().decode())
        self.h = h
        for o in observations:
            arrs = [np.ascontiguousarray(x, dtype=np.float64) if x is not None else None
                    for x in (o.centers_or_edges, o.data, o.error, o.weight, o.fwhm,
                              o.filter_wavelength, o.filter_response)]
            self._keep.append(arrs)
            ce, d, e, w, f, fw, fr = arrs
            nf = 0 if fw is None else fw.size
            rc = L.orc_add_observation(h, o.name.encode(), o.type.encode(), o.n, _ptr(ce), _ptr(d), _ptr(e),
                                       _ptr(w), _ptr(f), nf, _ptr(fw), _ptr(fr),
                                       (o.detector or "").encode(), (o.modifier or "").encode())
            if rc:
                raise RuntimeError("oracle: " + L.orc_last_error().decode())
        if L.orc_finalize(h):
            raise RuntimeError("oracle: " + L.orc_last_error().decode())
        self.N = L.orc_nb_spectral_points(h)
        self.M = L.orc_nb_obs_points(h)
        self.P = L.orc_nb_parameters(h)

    def close(self) -> None:
        """Frees the model's tables and operators (several GB at the largest workload)."""
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def grid(self) -> np.ndarray:
        out = np.empty(self.N)
        lib().orc_grid(self.h, _ptr(out))
        return out

    def forward(self, params):
        p = np.ascontiguousarray(params, dtype=np.float64)
        spec = np.empty(self.N)
        obs = np.empty(max(self.M, 1))
        neg = C.c_int(0)
        if lib().orc_forward(self.h, _ptr(p), p.size, _ptr(spec), _ptr(obs), C.byref(neg)):
            raise RuntimeError("oracle: " + lib().orc_last_error().decode())
        return spec, obs[: self.M], bool(neg.value)

    def contribution(self, params, levels: int):
        """Contribution functions: (levels x N high-resolution, levels x M binned)."""
        p = np.ascontiguousarray(params, dtype=np.float64)
        hr = np.empty((levels, self.N))
        bins = np.empty((levels, max(self.M, 1)))
        if lib().orc_contribution(self.h, _ptr(p), p.size, _ptr(hr), _ptr(bins)):
            raise RuntimeError("oracle: " + lib().orc_last_error().decode())
        return hr, bins[:, : self.M]

    def set_tau_cutoff(self, tau: float) -> None:
        """Optical depth at which transmission tangent sums stop (10, the reference's; inf: none)."""
        if lib().orc_set_tau_cutoff(self.h, float(tau)):
            raise RuntimeError("oracle: invalid cut-off")

    def loglike(self, params) -> float:
        p = np.ascontiguousarray(params, dtype=np.float64)
        out = C.c_double(0)
        if lib().orc_loglike(self.h, _ptr(p), p.size, C.byref(out), C.cast(None, _dp)):
            raise RuntimeError("oracle: " + lib().orc_last_error().decode())
        return out.value

    def obs_setup(self, k: int):
        cap = 4 * self.N + 16
        buf = (C.c_long * cap)()
        n = lib().orc_obs_setup(self.h, k, buf, cap)
        v = list(buf[:n])
        lo, hi, nb = v[0], v[1], v[2]
        edges = [(v[3 + 2 * i], v[4 + 2 * i]) for i in range(nb)]
        rest = v[3 + 2 * nb:]
        conv = [(rest[2 * i], rest[2 * i + 1]) for i in range(len(rest) // 2)]
        return {"range": (lo, hi), "edges": edges, "conv": conv}


def set_threads(n: int) -> int:
    return lib().orc_set_threads(int(n))
