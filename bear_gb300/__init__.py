"""GB300-native likelihood engine for BeAR's per-likelihood forward-model path.

The names mirror the reference's Python binding ``pybear``
(python/src/bear_python_wrapper.cpp): Config, Observation, Prior,
EmissionModelConfig, TransmissionModelConfig, OccultationConfig, Retrieval,
ForwardModelOutput, SpectralGrid. The compute runs in hand-written sm_103a kernels of
libbeargb300.so (C ABI: include/bear_gb300.h).
"""

from .config import (Config, EmissionModelConfig, GenericConfig, Observation, OccultationConfig, Prior,
                     TransmissionModelConfig, observation_arrays, render_config)
from .retrieval import Engine, ForwardModelOutput, Priors, Retrieval, SpectralGrid

__all__ = [
    "Config", "EmissionModelConfig", "GenericConfig", "Observation", "OccultationConfig", "Prior",
    "TransmissionModelConfig", "observation_arrays", "render_config", "Engine",
    "ForwardModelOutput", "Priors", "Retrieval", "SpectralGrid",
]
