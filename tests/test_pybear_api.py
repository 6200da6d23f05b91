"""bear_gb300's Python classes against pyBeAR's binding table.

tests/golden/pybear_api.json is extracted from the reference's
python/src/bear_python_wrapper.cpp by tests/golden/make_pybear_api.py. For every pyBeAR
class this package provides, each constructor overload's argument count must bind to
the class's signature, and every method and read/write field must exist. The classes
and overloads this package does not provide are listed below with the reason; the test
fails if the table names anything else that is missing."""

import inspect
import json
import os

import pytest

import bear_gb300
from bear_gb300 import config as cfg
from bear_gb300 import retrieval as ret

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE = json.load(open(os.path.join(HERE, "golden", "pybear_api.json")))["classes"]
NAMESPACE = {**vars(cfg), **vars(ret), **vars(bear_gb300)}

# pyBeAR classes outside this engine's scope (post-processing, MultiNest runs, the
# planet-blackbody eclipse and flat-line models, the stand-alone spectrum calculators)
NOT_PROVIDED = {
    "AtmosphereOutput": "atmosphere post-processing output",
    "PostProcess": "post-processing runs",
    "EmissionPostProcessConfig": "post-processing configuration",
    "TransmissionPostProcessConfig": "post-processing configuration",
    "OccultationPostProcessConfig": "post-processing configuration",
    "OccultationBlackBodyPostConfig": "post-processing configuration",
    "FlatLinePostProcessConfig": "post-processing configuration",
    "OccultationBlackBodyConfig": "planet-blackbody eclipse model (secondary_eclipse_bb)",
    "EmissionModel": "stand-alone spectrum calculator for a given atmosphere (calcSpectrum)",
    "TransmissionModel": "stand-alone spectrum calculator for a given atmosphere (calcSpectrum)",
    "OccultationModel": "stand-alone spectrum calculator for a given atmosphere (calcSpectrum)",
}
# (class, constructor argument count or method name): configuration-file folders are read
# by BeAR's own config parsers, and Retrieval.run drives MultiNest
NOT_PROVIDED_MEMBERS = {
    ("Config", "loadConfigFile"): "reads retrieval.config from a folder",
    ("EmissionModelConfig", 1): "reads forward_model.config from a folder",
    ("OccultationConfig", 1): "reads forward_model.config from a folder",
    ("TransmissionModelConfig", 1): "reads forward_model.config from a folder",
    ("Retrieval", 1): "reads the whole retrieval set-up from a folder",
    ("Retrieval", "run"): "MultiNest run (bear_gb300.sampler.BatchedNestedSampler is the batched driver)",
    ("Retrieval", "computeAtmosphereStructure"): "bound to a PostProcess member in pyBeAR; post-processing",
    ("SpectralGrid", 3): "grid from a GlobalConfig and bounds (the engine samples its own grid)",
}


# classes whose constructor takes *args (one Python signature for several C++ overloads)
CONSTRUCT = {
    "TransmissionModelConfig": {
        9: lambda: cfg.TransmissionModelConfig(50, 10.0, 1e-6, "const", [], ["iso"], [["H2O"]], ["H2O"], ["H2O"]),
        16: lambda: cfg.TransmissionModelConfig(False, False, False, 50, 10.0, 1e-6, "const", [], ["iso"], [["H2O"]],
                                                ["H2O"], ["H2O"], [], [], [], []),
    },
}


@pytest.mark.parametrize("name", sorted(TABLE))
def test_class_matches_pybear(name):
    entry = TABLE[name]
    if name in NOT_PROVIDED:
        return
    assert name in NAMESPACE and inspect.isclass(NAMESPACE[name]), f"pyBeAR class {name} is missing"
    cls = NAMESPACE[name]
    sig = inspect.signature(cls)
    for n in entry["init_arg_counts"]:
        if (name, n) in NOT_PROVIDED_MEMBERS:
            continue
        if n in CONSTRUCT.get(name, {}):
            CONSTRUCT[name][n]()  # a class taking *args: construct the overload for real
        else:
            sig.bind(*([None] * n))  # raises TypeError when the overload's arity is not accepted
    for m in entry["methods"]:
        if (name, m) in NOT_PROVIDED_MEMBERS:
            continue
        assert callable(getattr(cls, m, None)), f"{name}.{m} is missing"


def _instances():
    return {
        "Config": cfg.Config(True, "emission", "/tmp/x/", "const_wavenumber", 1.0, "", ""),
        "Observation": cfg.Observation("o", "spectroscopy", [1.0, 2.0], [1.0, 1.0], [0.1, 0.1]),
        "Prior": cfg.Prior("uniform", "a", [0.0, 1.0]),
        "ForwardModelOutput": ret.ForwardModelOutput(),
        "EmissionModelConfig": cfg.EmissionModelConfig(50, 100.0, 1e-3, "const", [], "scm", [], ["iso"], [["H2O"]],
                                                       ["H2O"], ["H2O"]),
        "TransmissionModelConfig": cfg.TransmissionModelConfig(50, 10.0, 1e-6, "const", [], ["iso"], [["H2O"]],
                                                               ["H2O"], ["H2O"]),
        "OccultationConfig": cfg.OccultationConfig(50, 100.0, 1e-3, "const", [], "scm", [], ["iso"], [["H2O"]],
                                                   ["H2O"], ["H2O"], "blackbody", []),
        "SpectralGrid": ret.SpectralGrid(__import__("numpy").array([1000.0, 1001.0])),
    }


@pytest.mark.parametrize("name", sorted(_instances()))
def test_fields_match_pybear(name):
    obj = _instances()[name]
    for f in TABLE[name]["fields"]:
        assert hasattr(obj, f), f"{name}.{f} is missing"
