"""pyBeAR-compatible configuration objects and their rendering to config text.

The classes keep the names, constructor argument orders and attribute names of
the reference's Python binding (python/src/bear_python_wrapper.cpp:28-300):
``Config`` (GlobalConfig, src/config/global_config.h:27-71), ``Observation``
(ObservationInput, src/observations/observations.h:42-92), ``Prior``
(PriorConfig, src/retrieval/priors.h:32-49), ``EmissionModelConfig``
(src/forward_model/emission/emission.h:44-100), ``TransmissionModelConfig``
(src/forward_model/transmission/transmission.h:47-110) and ``OccultationConfig``
(src/forward_model/secondary_eclipse/secondary_eclipse.h:53-105).

The engine itself is configured through a line-based ``key value...`` text
(``render_config``) plus per-observation arrays, which is what crosses the
C ABI (include/bear_gb300.h).
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

_DISCRETISATIONS = ("const_wavenumber", "const_wavelength", "const_resolution")


class Config:
    """GlobalConfig: src/config/global_config.h:27-71, 7-argument constructor
    src/config/global_config.cpp:37-74 (discretisation names checked there)."""

    def __init__(
        self,
        use_gpu: bool = True,
        forward_model_type: str = "",
        cross_section_file_path: str = "",
        spectral_disecretisation: str = "const_wavenumber",
        resolution: float = 1.0,
        multinest_output_path: str = "",
        post_output_path: str = "",
    ):
        if spectral_disecretisation not in _DISCRETISATIONS:
            raise ValueError(
                f"Spectral discretisation parameter: {spectral_disecretisation} unknown!"
            )
        self.use_gpu = bool(use_gpu)
        self.forward_model_type = forward_model_type
        self.cross_section_file_path = cross_section_file_path
        self.spectral_disecretisation = _DISCRETISATIONS.index(spectral_disecretisation)
        self.spectral_resolution = float(resolution)
        self.multinest_output_path = multinest_output_path
        self.post_output_path = post_output_path
        self.wavenumber_file_path = ""
        self.retrieval_folder_path = ""
        self.use_error_inflation = False
        self.multinest_print_iter_values = False
        self.multinest_efficiency = 0.8
        self.multinest_nb_living_points = 100
        self.multinest_nb_iterations = 0
        self.multinest_feedback = False
        self.nb_omp_processes = 0


class Observation:
    """ObservationInput: src/observations/observations.h:42-92."""

    def __init__(self, name: str = "", type: str = "", a=None, data=None, data_error=None):
        self.name = name
        self.type = type
        self.wavelengths: List[float] = []
        self.bin_wavelength_edges: List[List[float]] = []
        if a is not None:
            arr = np.asarray(a, dtype=np.float64)
            if arr.ndim == 1:
                self.wavelengths = list(arr)
            else:
                self.bin_wavelength_edges = [list(r) for r in arr]
        self.data = list(np.asarray(data if data is not None else [], dtype=np.float64))
        self.data_error = list(np.asarray(data_error if data_error is not None else [], dtype=np.float64))
        self.likelihood_weight: List[float] = []
        self.instrument_profile_fwhm: List[float] = []
        self.filter_response: List[List[float]] = []
        self.filter_detector_type = ""
        self.spectrum_modifier_id = ""

    def nb_points(self) -> int:
        return len(self.data)


@dataclass
class Prior:
    """PriorConfig: src/retrieval/priors.h:32-49."""

    type: str
    description: str
    parameter: Sequence[float]
    unit: str = ""


class GenericConfig:
    pass


class EmissionModelConfig(GenericConfig):
    """src/forward_model/emission/emission.h:44-100; constructor argument order of
    src/forward_model/emission/emission_model_config.cpp:79-110."""

    def __init__(
        self,
        nb_grid_points: int,
        atmos_bottom_pressure: float,
        atmos_top_pressure: float,
        temperature_profile_model: str,
        temperature_profile_parameters: Sequence[str],
        radiative_transfer_model: str,
        radiative_transfer_parameters: Sequence[str],
        chemistry_model: Sequence[str],
        chemistry_parameters: Sequence[Sequence[str]],
        opacity_species_symbol: Sequence[str],
        opacity_species_folder: Sequence[str],
        cloud_model: Sequence[str] = (),
        cloud_model_parameters: Sequence[Sequence[str]] = (),
    ):
        self.nb_grid_points = int(nb_grid_points)
        self.atmos_boundaries = [float(atmos_bottom_pressure), float(atmos_top_pressure)]
        self.temperature_profile_model = temperature_profile_model
        self.temperature_profile_parameters = list(temperature_profile_parameters)
        self.radiative_transfer_model = radiative_transfer_model
        self.radiative_transfer_parameters = list(radiative_transfer_parameters)
        self.chemistry_model = list(chemistry_model)
        self.chemistry_parameters = [list(p) for p in chemistry_parameters]
        self.opacity_species_symbol = list(opacity_species_symbol)
        self.opacity_species_folder = list(opacity_species_folder)
        self.cloud_model = list(cloud_model)
        self.cloud_model_parameters = [list(p) for p in cloud_model_parameters]

    forward_model_type = "emission"


class TransmissionModelConfig(GenericConfig):
    """src/forward_model/transmission/transmission.h:47-110 (both constructors)."""

    forward_model_type = "transmission"

    def __init__(self, *args):
        if isinstance(args[0], (bool, np.bool_)) and len(args) == 16:
            (fit_mmw, fit_sh, var_g, nb, pb, pt, tm, tp, cm, cp, os_, of, cl, clp, mods, modp) = args
        elif len(args) == 9:
            (nb, pb, pt, tm, tp, cm, cp, os_, of) = args
            fit_mmw = fit_sh = var_g = False
            cl, clp, mods, modp = [], [], [], []
        else:
            raise TypeError("TransmissionModelConfig: unsupported constructor arguments")
        self.fit_mean_molecular_weight = bool(fit_mmw)
        self.fit_scale_height = bool(fit_sh)
        self.use_variable_gravity = bool(var_g)
        self.nb_grid_points = int(nb)
        self.atmos_boundaries = [float(pb), float(pt)]
        self.temperature_profile_model = tm
        self.temperature_profile_parameters = list(tp)
        self.chemistry_model = list(cm)
        self.chemistry_parameters = [list(p) for p in cp]
        self.opacity_species_symbol = list(os_)
        self.opacity_species_folder = list(of)
        self.cloud_model = list(cl)
        self.cloud_model_parameters = [list(p) for p in clp]
        self.modules = list(mods)
        self.modules_parameters = [list(p) for p in modp]
        # impact parameters per atmospheric layer (not in the reference: 1 is its tangent
        # ray per level; A > 1 adds A - 1 rays inside every layer, extinction linear in z)
        self.transmission_annuli = 1


class OccultationConfig(GenericConfig):
    """Secondary-eclipse model, src/forward_model/secondary_eclipse/secondary_eclipse.h:53-105;
    constructor argument order of secondary_eclipse_model_config.cpp:76-112 (the one pyBeAR
    binds, python/src/bear_python_wrapper.cpp:203-221), clouds optional.

    stellar_spectrum_model: "blackbody" (no parameters; T_eff is fitted), "file" [path]
    ("wavelength flux" lines, W m^-2 um^-1) or "grid" [folder/] (T_eff, log g, [M/H] fitted)."""

    forward_model_type = "secondary_eclipse"

    def __init__(
        self,
        nb_grid_points: int,
        atmos_bottom_pressure: float,
        atmos_top_pressure: float,
        temperature_profile_model: str,
        temperature_profile_parameters: Sequence[str],
        radiative_transfer_model: str,
        radiative_transfer_parameters: Sequence[str],
        chemistry_model: Sequence[str],
        chemistry_parameters: Sequence[Sequence[str]],
        opacity_species_symbol: Sequence[str],
        opacity_species_folder: Sequence[str],
        stellar_spectrum_model: str,
        stellar_model_parameters: Sequence[str],
        cloud_model: Sequence[str] = (),
        cloud_model_parameters: Sequence[Sequence[str]] = (),
    ):
        self.nb_grid_points = int(nb_grid_points)
        self.atmos_boundaries = [float(atmos_bottom_pressure), float(atmos_top_pressure)]
        self.temperature_profile_model = temperature_profile_model
        self.temperature_profile_parameters = list(temperature_profile_parameters)
        self.radiative_transfer_model = radiative_transfer_model
        self.radiative_transfer_parameters = list(radiative_transfer_parameters)
        self.chemistry_model = list(chemistry_model)
        self.chemistry_parameters = [list(p) for p in chemistry_parameters]
        self.opacity_species_symbol = list(opacity_species_symbol)
        self.opacity_species_folder = list(opacity_species_folder)
        self.stellar_spectrum_model = stellar_spectrum_model
        self.stellar_model_parameters = list(stellar_model_parameters)
        self.cloud_model = list(cloud_model)
        self.cloud_model_parameters = [list(p) for p in cloud_model_parameters]


def _fmt(x: float) -> str:
    return repr(float(x))


def _ensure_slash(p: str) -> str:
    return p if (p == "" or p.endswith("/")) else p + "/"


def render_config(config: Config, model_config: GenericConfig) -> str:
    """Render the engine's line-based configuration text."""
    mt = getattr(model_config, "forward_model_type", config.forward_model_type)
    lines = [
        f"forward_model {mt}",
        f"cross_section_path {_ensure_slash(config.cross_section_file_path)}",
        f"wavenumber_file {config.wavenumber_file_path}",
        f"spectral_discretisation {_DISCRETISATIONS[config.spectral_disecretisation]}",
        f"spectral_resolution {_fmt(config.spectral_resolution)}",
        f"error_inflation {1 if config.use_error_inflation else 0}",
        f"nb_grid_points {model_config.nb_grid_points}",
        "atmos_boundaries {} {}".format(*[_fmt(x) for x in model_config.atmos_boundaries]),
        " ".join(["temperature_profile", model_config.temperature_profile_model]
                 + list(model_config.temperature_profile_parameters)),
    ]
    if mt in ("emission", "secondary_eclipse", "Secondary_eclipse", "se"):
        lines.append(" ".join(["radiative_transfer", model_config.radiative_transfer_model]
                              + list(model_config.radiative_transfer_parameters)))
        if mt != "emission":
            lines.append(" ".join(["stellar_spectrum", model_config.stellar_spectrum_model]
                                  + list(model_config.stellar_model_parameters)))
    else:
        lines.append(f"fit_mean_molecular_weight {int(model_config.fit_mean_molecular_weight)}")
        lines.append(f"fit_scale_height {int(model_config.fit_scale_height)}")
        lines.append(f"variable_gravity {int(model_config.use_variable_gravity)}")
        if getattr(model_config, "modules", []):
            raise ValueError("transmission spectrum modules are not supported by this engine")
        annuli = int(getattr(model_config, "transmission_annuli", 1))
        if annuli != 1:
            lines.append(f"transmission_annuli {annuli}")
    for m, p in zip(model_config.chemistry_model, model_config.chemistry_parameters):
        lines.append(" ".join(["chemistry", m] + list(p)))
    for m, p in zip(model_config.cloud_model, model_config.cloud_model_parameters):
        lines.append(" ".join(["cloud", m] + list(p)))
    for s, f in zip(model_config.opacity_species_symbol, model_config.opacity_species_folder):
        lines.append(f"opacity {s} {f}" if f else f"opacity {s}")
    return "\n".join(lines) + "\n"


@dataclass
class ObservationArrays:
    """Flattened observation as it crosses the C ABI."""

    name: str
    type: str
    n: int
    centers_or_edges: np.ndarray  # (n,) for spectroscopy, (n, 2) otherwise
    data: np.ndarray
    error: np.ndarray
    weight: Optional[np.ndarray]
    fwhm: Optional[np.ndarray]
    filter_wavelength: Optional[np.ndarray]
    filter_response: Optional[np.ndarray]
    detector: str
    modifier: str


def observation_arrays(o: Observation) -> ObservationArrays:
    t = o.type
    if t in ("spectroscopy", "Spectroscopy"):
        ce = np.ascontiguousarray(o.wavelengths, dtype=np.float64)
    else:
        ce = np.ascontiguousarray(o.bin_wavelength_edges, dtype=np.float64).reshape(-1, 2)
    n = len(o.data)
    fw = np.ascontiguousarray(o.instrument_profile_fwhm, dtype=np.float64) if len(o.instrument_profile_fwhm) else None
    wt = np.ascontiguousarray(o.likelihood_weight, dtype=np.float64) if len(o.likelihood_weight) else None
    fl_w = fl_r = None
    if len(o.filter_response):
        fl_w = np.ascontiguousarray(o.filter_response[0], dtype=np.float64)
        fl_r = np.ascontiguousarray(o.filter_response[1], dtype=np.float64)
    return ObservationArrays(
        name=o.name, type=t, n=n, centers_or_edges=ce,
        data=np.ascontiguousarray(o.data, dtype=np.float64),
        error=np.ascontiguousarray(o.data_error, dtype=np.float64),
        weight=wt, fwhm=fw, filter_wavelength=fl_w, filter_response=fl_r,
        detector=o.filter_detector_type or "", modifier=o.spectrum_modifier_id or "",
    )
