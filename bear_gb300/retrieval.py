"""pyBeAR-compatible front end of the GB300 engine.

``Retrieval(config, model_config, observations, priors)`` keeps the names and
semantics of the reference's binding (python/src/bear_python_wrapper.cpp:114-129):
``computeLikelihood``, ``computeModel``, ``convertCubeParameters``,
``convertToPhysicalParameters``, ``nbParameters`` and ``spectral_grid``. It adds
``computeLikelihoodBatch`` / ``computeGradientBatch`` for batches of parameter
sets evaluated in one launch, and ``BatchEvaluator`` that replays a captured
CUDA graph for a fixed batch size.
"""

from __future__ import annotations

import ctypes as C
import math
import weakref
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from .config import (Config, GenericConfig, Observation, ObservationArrays, Prior,
                     observation_arrays, render_config)

PARSEC = 3.08567758135e18
UNITS = {
    "": 1.0,
    "Me": 5.97219e27, "Mearth": 5.97219e27, "Mj": 1.89813e30, "Mjupiter": 1.89813e30,
    "Ms": 1.9884e33, "Msun": 1.9884e33, "Re": 6.37123e8, "Rearth": 6.37123e8,
    "Rj": 7.1492e9, "Rjupiter": 7.1492e9, "Rs": 6.96342e10, "Rsun": 6.96342e10,
    "ly": 9.4607304725808e17, "pc": PARSEC,
}


class Engine:
    """One device model: config text + observation arrays -> likelihood engine."""

    def __init__(self, config_text: str, observations: Sequence[ObservationArrays], device: int = 0,
                 prepare_only: bool = False):
        """prepare_only: run the host-side set-up (grid, observation operators,
        tables) without a GPU; evaluations are then unavailable."""
        lib = _lib.load()
        h = C.c_void_p()
        _lib.check(lib.bear_model_create(config_text.encode(), int(device), C.byref(h)))
        self._h = h
        self._graphs = weakref.WeakSet()  # captured batches to destroy before the model
        self._lib = lib
        self.device = int(device)
        self._keep = []
        try:
            for o in observations:
                arrs = [None if x is None else np.ascontiguousarray(x, dtype=np.float64)
                        for x in (o.centers_or_edges, o.data, o.error, o.weight, o.fwhm,
                                  o.filter_wavelength, o.filter_response)]
                ce, d, e, w, f, fw, fr = arrs
                self._keep.append(arrs)
                nf = 0 if fw is None else int(fw.size)
                _lib.check(lib.bear_model_add_observation(
                    h, o.name.encode(), o.type.encode(), int(o.n), _lib.dptr(ce), _lib.dptr(d), _lib.dptr(e),
                    _lib.dptr(w), _lib.dptr(f), nf, _lib.dptr(fw), _lib.dptr(fr),
                    (o.detector or "").encode(), (o.modifier or "").encode()))
            _lib.check(lib.bear_model_prepare(h) if prepare_only else lib.bear_model_finalize(h))
            self.finalized = not prepare_only
        except Exception:
            lib.bear_model_destroy(h)
            self._h = None
            raise
        N, M, P, K = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        _lib.check(lib.bear_model_info(h, C.byref(N), C.byref(M), C.byref(P), C.byref(K)))
        self.N, self.M, self.P, self.nobs = N.value, M.value, P.value, K.value
        self.obs_sizes = []
        for k in range(self.nobs):
            n = C.c_int()
            _lib.check(lib.bear_model_observation_size(h, k, C.byref(n)))
            self.obs_sizes.append(n.value)
        self.wavenumbers = np.empty(self.N)
        _lib.check(lib.bear_model_wavenumbers(h, _lib.dptr(self.wavenumbers)))

    def observation_setup(self, k: int) -> dict:
        """Integer set-up of observation k: observation index range, band-edge
        indices and convolution windows (as SpectralBands holds them)."""
        cap = 4 * self.N + 16
        buf = (C.c_longlong * cap)()
        n = C.c_int()
        _lib.check(self._lib.bear_model_observation_setup(self._h, int(k), buf, cap, C.byref(n)))
        v = list(buf[: n.value])
        nb = v[2]
        edges = [(v[3 + 2 * i], v[4 + 2 * i]) for i in range(nb)]
        rest = v[3 + 2 * nb:]
        conv = [(rest[2 * i], rest[2 * i + 1]) for i in range(len(rest) // 2)]
        return {"range": (v[0], v[1]), "edges": edges, "conv": conv}

    def operator_row(self, r: int):
        """(k0, weights) of row r of the composite observation operator."""
        k0, ln = C.c_int(), C.c_int()
        w = C.POINTER(C.c_double)()
        _lib.check(self._lib.bear_model_operator_row(self._h, int(r), C.byref(k0), C.byref(ln), C.byref(w)))
        return k0.value, np.ctypeslib.as_array(w, shape=(ln.value,)).copy()

    # ------------------------------------------------------------ plain path
    def _params(self, params) -> np.ndarray:
        p = np.ascontiguousarray(params, dtype=np.float64).ravel()
        if p.size != self.P:
            raise ValueError(f"expected {self.P} parameters, got {p.size}")
        return p

    def compute_model(self, params, stream: int = 0):
        p = self._params(params)
        spec = np.empty(self.N)
        obs = np.empty(max(self.M, 1))
        neg = C.c_int(0)
        _lib.check(self._lib.bear_compute_model(self._h, _lib.dptr(p), p.size, _lib.dptr(spec), _lib.dptr(obs),
                                                C.byref(neg), C.c_void_p(stream)))
        return spec, obs[: self.M], bool(neg.value)

    def contribution_functions(self, params, stream: int = 0):
        """Contribution functions of one parameter set (emission and secondary-eclipse
        models): (binned, levels x M in compute_model's observation order; high-resolution,
        levels x N). Level 0 is the bottom of the atmosphere."""
        p = self._params(params)
        L = self.table_info()["levels"]
        bins = np.empty((L, max(self.M, 1)))
        hr = np.empty((L, self.N))
        _lib.check(self._lib.bear_contribution_functions(self._h, _lib.dptr(p), p.size, _lib.dptr(bins),
                                                         _lib.dptr(hr), C.c_void_p(stream)))
        return bins[:, : self.M], hr

    def loglike(self, params, stream: int = 0) -> float:
        p = self._params(params)
        out = C.c_double(0.0)
        _lib.check(self._lib.bear_loglike(self._h, _lib.dptr(p), p.size, C.byref(out), C.c_void_p(stream)))
        return out.value

    def forward_device(self, params, spectrum_ptr: int, obs_ptrs: Optional[Sequence[int]], stream: int = 0) -> bool:
        """ForwardModel::calcModelGPU: device outputs given as raw pointers."""
        p = self._params(params)
        arr = None
        if obs_ptrs is not None:
            arr = (C.POINTER(C.c_double) * self.nobs)(*[C.cast(C.c_void_p(x), C.POINTER(C.c_double)) for x in obs_ptrs])
        neg = C.c_int(0)
        _lib.check(self._lib.bear_forward(self._h, _lib.dptr(p), p.size,
                                          C.cast(C.c_void_p(spectrum_ptr), C.POINTER(C.c_double)) if spectrum_ptr else C.cast(None, C.POINTER(C.c_double)),
                                          arr, C.byref(neg), C.c_void_p(stream)))
        return bool(neg.value)

    # ------------------------------------------------------------ batched path
    def loglike_batch_ptr(self, params_ptr: int, batch: int, loglike_ptr: int, neglect_ptr: int = 0,
                          stream: int = 0) -> None:
        _lib.check(self._lib.bear_loglike_batch(self._h, C.c_void_p(params_ptr), int(batch), self.P,
                                                C.c_void_p(loglike_ptr), C.c_void_p(neglect_ptr or None),
                                                C.c_void_p(stream)))

    def grad_batch_ptr(self, params_ptr: int, batch: int, loglike_ptr: int, grad_ptr: int,
                       neglect_ptr: int = 0, stream: int = 0) -> None:
        _lib.check(self._lib.bear_loglike_grad_batch(self._h, C.c_void_p(params_ptr), int(batch), self.P,
                                                     C.c_void_p(loglike_ptr), C.c_void_p(grad_ptr),
                                                     C.c_void_p(neglect_ptr or None), C.c_void_p(stream)))

    def loglike_batch(self, params):
        """params: torch float64 CUDA tensor (B, P). Returns (loglike (B,), neglect (B,) uint8)."""
        import torch
        t = params.contiguous()
        assert t.dtype == torch.float64 and t.is_cuda and t.shape[1] == self.P
        B = t.shape[0]
        ll = torch.empty(B, dtype=torch.float64, device=t.device)
        ng = torch.empty(B, dtype=torch.uint8, device=t.device)
        self.loglike_batch_ptr(t.data_ptr(), B, ll.data_ptr(), ng.data_ptr(),
                               torch.cuda.current_stream(t.device).cuda_stream)
        return ll, ng

    # ------------------------------------------------------------ priors on the device
    _PRIOR_TYPES = {"uniform": 0, "log_uniform": 1, "gaussian": 2, "delta": 3, "linked": 4}

    def set_priors(self, priors: Sequence[Prior]) -> None:
        """Upload one prior per parameter (pyBeAR Prior objects; "linked" priors take the
        1-based index of the parameter they follow, as the reference's config)."""
        n = len(priors)
        typ = np.zeros(n, dtype=np.int32)
        a, b, u = np.zeros(n), np.zeros(n), np.ones(n)
        link = np.full(n, -1, dtype=np.int32)
        for i, p in enumerate(priors):
            if p.type not in self._PRIOR_TYPES:
                raise ValueError(f"Prior type {p.type} for {p.description} unknown!")
            typ[i] = self._PRIOR_TYPES[p.type]
            if p.type == "linked":
                link[i] = int(p.parameter[0]) - 1
                continue
            a[i] = p.parameter[0]
            b[i] = p.parameter[1] if len(p.parameter) > 1 else 0.0
            if p.unit not in UNITS:
                raise ValueError(f"Unit {p.unit} for parameter {p.description} unknown!")
            u[i] = UNITS[p.unit]
        ip = C.POINTER(C.c_int)
        _lib.check(self._lib.bear_model_set_priors(self._h, n, typ.ctypes.data_as(ip), _lib.dptr(a), _lib.dptr(b),
                                                   _lib.dptr(u), link.ctypes.data_as(ip)))

    def prior_transform_batch(self, cube):
        """cube: torch float64 CUDA tensor (B, P) in [0, 1]. Returns the physical parameters."""
        import torch
        t = cube.contiguous()
        assert t.dtype == torch.float64 and t.is_cuda and t.shape[1] == self.P
        out = torch.empty_like(t)
        _lib.check(self._lib.bear_prior_transform_batch(self._h, C.c_void_p(t.data_ptr()), t.shape[0], self.P,
                                                        C.c_void_p(out.data_ptr()),
                                                        C.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)))
        return out

    def loglike_cube_batch(self, cube):
        """cube: torch float64 CUDA tensor (B, P). Returns (loglike, neglect, physical parameters)."""
        import torch
        t = cube.contiguous()
        assert t.dtype == torch.float64 and t.is_cuda and t.shape[1] == self.P
        B = t.shape[0]
        par = torch.empty_like(t)
        ll = torch.empty(B, dtype=torch.float64, device=t.device)
        ng = torch.empty(B, dtype=torch.uint8, device=t.device)
        _lib.check(self._lib.bear_loglike_cube_batch(self._h, C.c_void_p(t.data_ptr()), B, self.P,
                                                     C.c_void_p(par.data_ptr()), C.c_void_p(ll.data_ptr()),
                                                     C.c_void_p(ng.data_ptr()),
                                                     C.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)))
        return ll, ng, par

    def grad_batch(self, params):
        """params: torch float64 CUDA tensor (B, P). Returns (loglike (B,), d loglike / d params
        (B, P), neglect (B,) uint8) from the adjoint kernels."""
        import torch
        t = params.detach().contiguous()
        assert t.dtype == torch.float64 and t.is_cuda and t.shape[1] == self.P
        B = t.shape[0]
        ll = torch.empty(B, dtype=torch.float64, device=t.device)
        g = torch.empty(B, self.P, dtype=torch.float64, device=t.device)
        ng = torch.empty(B, dtype=torch.uint8, device=t.device)
        self.grad_batch_ptr(t.data_ptr(), B, ll.data_ptr(), g.data_ptr(), ng.data_ptr(),
                            torch.cuda.current_stream(t.device).cuda_stream)
        return ll, g, ng

    def set_precision(self, mode: int) -> None:
        """0: double-float opacity assembly (default); 1: every step in FP64."""
        _lib.check(self._lib.bear_model_set_precision(self._h, int(mode)))

    def autotune(self, params) -> int:
        """Time the radiative-transfer launch shapes on ``params`` (torch float64 CUDA,
        (B, P), B >= 2) and keep the fastest for batched calls; returns it."""
        import torch
        t = params.detach().contiguous()
        assert t.dtype == torch.float64 and t.is_cuda and t.shape[1] == self.P
        best = C.c_int()
        _lib.check(self._lib.bear_model_autotune(self._h, C.c_void_p(t.data_ptr()), int(t.shape[0]), self.P,
                                                 C.c_void_p(torch.cuda.current_stream(t.device).cuda_stream),
                                                 C.byref(best)))
        return best.value

    def table_sharing(self) -> Tuple[bool, int]:
        """(tables shared with another model on this device, their device bytes)."""
        sh, nb = C.c_int(), C.c_size_t()
        _lib.check(self._lib.bear_model_table_sharing(self._h, C.byref(sh), C.byref(nb)))
        return bool(sh.value), int(nb.value)

    def set_tau_cutoff(self, tau: float = 10.0) -> None:
        """Optical depth at which transmission tangent sums stop (10, the reference's; inf: none)."""
        _lib.check(self._lib.bear_model_set_tau_cutoff(self._h, float(tau)))

    def set_gradient_memory(self, nbytes: int = 0) -> None:
        """Device memory the gradient's work buffers may use per chunk (0 = default)."""
        _lib.check(self._lib.bear_model_set_gradient_memory(self._h, int(nbytes)))

    def set_launch(self, rt_threads: int = 0, obs_threads: int = 0) -> None:
        _lib.check(self._lib.bear_model_set_launch(self._h, int(rt_threads), int(obs_threads)))

    def table_info(self) -> dict:
        L, S, R, rows = C.c_int(), C.c_int(), C.c_int(), C.c_longlong()
        _lib.check(self._lib.bear_model_table_info(self._h, C.byref(L), C.byref(S), C.byref(R), C.byref(rows)))
        return {"levels": L.value, "table_species": S.value, "rayleigh_species": R.value, "rows": rows.value}

    @property
    def table_species(self) -> int:
        return self.table_info()["table_species"]

    def stencil_row_count(self, batch: int = 1) -> int:
        """Distinct table rows referenced by the last `batch` evaluations."""
        n = C.c_longlong()
        _lib.check(self._lib.bear_model_stencil_rows(self._h, int(batch), C.byref(n)))
        return n.value

    def stage_times(self, params_ptr: int, batch: int, loglike_ptr: int, stream: int = 0, repeats: int = 3):
        """Per-stage device times (ms) of a batched evaluation: atmosphere,
        radiative transfer, observation operator + likelihood (median of repeats)."""
        _lib.check(self._lib.bear_model_set_profiling(self._h, 1))
        out = []
        try:
            for _ in range(repeats):
                self.loglike_batch_ptr(params_ptr, batch, loglike_ptr, 0, stream)
                ms = (C.c_float * 3)()
                _lib.check(self._lib.bear_model_stage_times(self._h, ms))
                out.append(list(ms))
        finally:
            _lib.check(self._lib.bear_model_set_profiling(self._h, 0))
        out = np.array(out)
        return [float(np.median(out[:, i])) for i in range(3)]

    def device_bytes(self) -> int:
        b = C.c_size_t()
        _lib.check(self._lib.bear_model_device_bytes(self._h, C.byref(b)))
        return b.value

    def close(self) -> None:
        for g in list(getattr(self, "_graphs", ())):
            g.close()
        if getattr(self, "_h", None):
            self._lib.bear_model_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchEvaluator:
    """Batched log-likelihoods through a captured CUDA graph.

    Owns device buffers for ``batch`` parameter sets; on creation optionally
    autotunes the engine's launch shape on ``params`` (B, P) and captures the
    kernel sequence once. Each call copies the new parameters into the owned
    buffer and replays the graph on the current stream; the returned tensors are
    the owned log-likelihood / neglect buffers (overwritten by the next call)."""

    def __init__(self, engine: "Engine", params, autotune: bool = True):
        import torch
        t = params.detach().contiguous()
        assert t.dtype == torch.float64 and t.is_cuda and t.shape[1] == engine.P
        self.engine = engine
        self.batch = int(t.shape[0])
        self.params = t.clone()
        self.loglike = torch.empty(self.batch, dtype=torch.float64, device=t.device)
        self.neglect = torch.empty(self.batch, dtype=torch.uint8, device=t.device)
        self.rt_threads = engine.autotune(self.params) if autotune and self.batch >= 2 else 0
        torch.cuda.synchronize(t.device)
        h = C.c_void_p()
        _lib.check(engine._lib.bear_batch_graph_create(engine._h, C.c_void_p(self.params.data_ptr()), self.batch,
                                                       engine.P, C.c_void_p(self.loglike.data_ptr()),
                                                       C.c_void_p(self.neglect.data_ptr()), C.byref(h)))
        self._g = h
        engine._graphs.add(self)

    def launch(self, stream: int = 0) -> None:
        """Replay the graph on the parameters currently in ``self.params``."""
        _lib.check(self.engine._lib.bear_batch_graph_launch(self._g, C.c_void_p(stream)))

    def __call__(self, params=None):
        import torch
        if params is not None:
            self.params.copy_(params, non_blocking=True)
        self.launch(torch.cuda.current_stream(self.params.device).cuda_stream)
        return self.loglike, self.neglect

    def close(self) -> None:
        if getattr(self, "_g", None):
            _lib.check(self.engine._lib.bear_batch_graph_destroy(self._g))
            self._g = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class ForwardModelOutput:
    """src/forward_model/forward_model.h:42-46"""

    neglect_model: bool = False
    spectrum: List[float] = field(default_factory=list)
    spectrum_obs: List[List[float]] = field(default_factory=list)


class SpectralGrid:
    """The parts of SpectralGrid the binding exposes (src/spectral_grid/spectral_grid.h:41-63)."""

    def __init__(self, wavenumbers: np.ndarray):
        self.wavenumber_list = list(wavenumbers)
        self.wavelength_list = list(1.0 / np.asarray(wavenumbers) * 1e4)

    @staticmethod
    def wavelengthToWavenumber(wavelength: float) -> float:
        return 1.0 / wavelength * 1e4


def _erfinv(y: float) -> float:
    from scipy.special import erfinv
    return float(erfinv(y))


class Priors:
    """Prior transforms of src/retrieval/prior_types.h:89-256 (uniform, log-uniform,
    Gaussian, delta, linked) with the unit factors of :57-82. A linked prior
    (parameter = 1-based index of another, non-linked parameter; Priors::setupLinkedPriors
    src/retrieval/priors.cpp:246-280) takes that parameter's prior at that parameter's
    cube coordinate and carries no unit (Retrieval::convertHypercubeParameters
    src/retrieval/multinest_loglike.cpp:59-97)."""

    def __init__(self, priors: Sequence[Prior]):
        self.priors = list(priors)
        self.links = [-1] * len(self.priors)
        for i, p in enumerate(self.priors):
            if p.type not in ("uniform", "log_uniform", "gaussian", "delta", "linked"):
                raise ValueError(f"Prior type {p.type} for {p.description} unknown!")
            if p.type == "linked":
                j = int(p.parameter[0]) - 1
                if not 0 <= j < len(self.priors):
                    raise ValueError(f"Linked prior {p.description} wrong index for link!")
                if self.priors[j].type == "linked":
                    raise ValueError(f"Linked prior {p.description} Can not link prior to another linked prior!")
                self.links[i] = j
            elif p.unit not in UNITS:
                raise ValueError(f"Unit {p.unit} for parameter {p.description} unknown!")

    def __len__(self):
        return len(self.priors)

    def cube_to_parameters(self, cube: Sequence[float]) -> List[float]:
        out = []
        for i, p in enumerate(self.priors):
            u = cube[i]
            if self.links[i] >= 0:
                p, u = self.priors[self.links[i]], cube[self.links[i]]
            if p.type == "uniform":
                lo, hi = sorted(p.parameter)
                out.append(lo + u * (hi - lo))
            elif p.type == "log_uniform":
                lo, hi = sorted([math.log10(p.parameter[0]), math.log10(p.parameter[1])])
                out.append(10.0 ** (lo + u * (hi - lo)))
            elif p.type == "gaussian":
                out.append(p.parameter[0] + p.parameter[1] * math.sqrt(2.0) * _erfinv(2.0 * u - 1.0))
            else:
                out.append(p.parameter[0])
        return out

    def to_physical(self, params: Sequence[float]) -> List[float]:
        return [v * (1.0 if p.type == "linked" else UNITS[p.unit]) for p, v in zip(self.priors, params)]

    def cube_to_physical_batch(self, cube: np.ndarray) -> np.ndarray:
        cube = np.atleast_2d(np.asarray(cube, dtype=np.float64))
        out = np.empty_like(cube)
        for j, p in enumerate(self.priors):
            c = cube[:, j]
            u = UNITS[p.unit] if p.type != "linked" else 1.0
            if self.links[j] >= 0:
                p, c = self.priors[self.links[j]], cube[:, self.links[j]]
            if p.type == "uniform":
                lo, hi = sorted(p.parameter)
                out[:, j] = (lo + c * (hi - lo)) * u
            elif p.type == "log_uniform":
                lo, hi = sorted(np.log10(p.parameter))
                out[:, j] = np.power(10.0, lo + c * (hi - lo)) * u
            elif p.type == "gaussian":
                from scipy.special import erfinv
                out[:, j] = (p.parameter[0] + p.parameter[1] * np.sqrt(2.0) * erfinv(2.0 * c - 1.0)) * u
            else:
                out[:, j] = p.parameter[0] * u
        return out


class Retrieval:
    """Retrieval(GlobalConfig*, GenericConfig*, vector<ObservationInput>, vector<PriorConfig>)
    (src/retrieval/retrieval.cpp:70-104) on the GB300 engine."""

    def __init__(self, config: Config, model_config: GenericConfig, observations: Sequence[Observation],
                 priors: Sequence[Prior], device: int = 0):
        self.config = config
        self.model_config = model_config
        self.observations = list(observations)
        self._arrays = [observation_arrays(o) for o in self.observations]
        self.engine = Engine(render_config(config, model_config), self._arrays, device)
        self.priors = Priors(priors)
        if len(self.priors) != self.engine.P:
            raise ValueError(f"Found {len(self.priors)} priors config but expected {self.engine.P}")
        if self.engine.finalized:
            self.engine.set_priors(self.priors.priors)
        self.spectral_grid = SpectralGrid(self.engine.wavenumbers)
        self.nb_observations = self.engine.nobs

    def nbParameters(self) -> int:
        return len(self.priors)

    def convertCubeParameters(self, cube: Sequence[float]) -> Tuple[List[float], List[float]]:
        params = self.priors.cube_to_parameters(cube)
        return params, self.priors.to_physical(params)

    def convertToPhysicalParameters(self, params: Sequence[float]) -> List[float]:
        return self.priors.to_physical(params)

    def computeLikelihood(self, physical_parameters: Sequence[float]) -> float:
        return self.engine.loglike(physical_parameters)

    def computeModel(self, physical_parameters: Sequence[float], return_high_res_spectrum: bool) -> ForwardModelOutput:
        spec, obs, neg = self.engine.compute_model(physical_parameters)
        out = ForwardModelOutput(neglect_model=neg)
        out.spectrum = list(spec) if return_high_res_spectrum else []
        off = 0
        for n in self.engine.obs_sizes:
            out.spectrum_obs.append(list(obs[off:off + n]))
            off += n
        return out

    def computeLikelihoodCubeBatch(self, cube):
        """Log L of a batch of hypercube points (B x P, a torch CUDA tensor or an array):
        the prior transform runs on the device. Returns (log L, physical parameters) as
        torch tensors on the device."""
        import torch
        t = torch.as_tensor(cube, dtype=torch.float64)
        if not t.is_cuda:
            t = t.to(f"cuda:{self.engine.device}")
        ll, ng, par = self.engine.loglike_cube_batch(t)
        return ll, par

    def computeLikelihoodBatch(self, physical_parameters) -> np.ndarray:
        import torch
        t = torch.as_tensor(np.asarray(physical_parameters, dtype=np.float64), device=f"cuda:{self.engine.device}")
        ll, _ = self.engine.loglike_batch(t)
        return ll.cpu().numpy()

    def computeGradientBatch(self, physical_parameters) -> Tuple[np.ndarray, np.ndarray]:
        import torch
        t = torch.as_tensor(np.asarray(physical_parameters, dtype=np.float64), device=f"cuda:{self.engine.device}")
        ll, g, _ = self.engine.grad_batch(t)
        return ll.cpu().numpy(), g.cpu().numpy()
