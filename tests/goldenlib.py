"""Golden-case helpers shared by the tests and tests/golden/make_golden.py.

A golden case is one .npz under tests/golden/ holding
  meta        JSON: workload spec, config-text template ({ROOT} = table
              directory), observation names/types/detectors/modifiers
  obs{i}_*    observation arrays (centers/edges, data, error, weight, fwhm, filter)
  params      S x P physical parameter sets
  ref_*       outputs of the reference's own CPU path (oracle/_ref) on them:
              ref_loglike (S), ref_neglect (S), ref_obs (S x M, caller order),
              ref_spectrum (rows listed in spectrum_rows x N), ref_grid (N)
  ref_setup_* per-observation integer set-up (index range, band edges, windows)
  star_*      secondary-eclipse cases: the stellar spectrum file (star_wl, star_flux)
              or stellar grid (star_axis0..2, star_grid_wl, star_grid_spectra) the
              config template names as {STAR}; meta "star" is "file" or "grid"
The tables are regenerated from the spec (bear_gb300.synthetic, bit-identical
on every platform) into a temporary directory, the star files from the arrays.
"""

from __future__ import annotations

import dataclasses
import glob
import json
import os
import tempfile
from typing import Dict, List, Tuple

import numpy as np

from bear_gb300 import synthetic as syn
from bear_gb300.config import ObservationArrays

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TABLE_ROOT = os.environ.get("BEAR_SYNTH_DIR", os.path.join(tempfile.gettempdir(), "bear_gb300_synth"))


def spec_from_meta(meta: dict) -> syn.WorkloadSpec:
    d = dict(meta["spec"])
    d["table"] = syn.TableSpec(**d["table"])
    d["rayleigh"] = tuple(d["rayleigh"])
    return syn.WorkloadSpec(**d)


def spec_to_meta(spec: syn.WorkloadSpec) -> dict:
    return dataclasses.asdict(spec)


def save_case(path: str, meta: dict, obs: List[ObservationArrays], params: np.ndarray, ref: dict) -> None:
    arrays = {"params": np.asarray(params, dtype=np.float64)}
    meta = dict(meta)
    meta["observations"] = []
    for i, o in enumerate(obs):
        meta["observations"].append({"name": o.name, "type": o.type, "n": o.n, "detector": o.detector,
                                     "modifier": o.modifier})
        arrays[f"obs{i}_ce"] = o.centers_or_edges
        arrays[f"obs{i}_data"] = o.data
        arrays[f"obs{i}_error"] = o.error
        for key, val in (("weight", o.weight), ("fwhm", o.fwhm), ("fwl", o.filter_wavelength),
                         ("fresp", o.filter_response)):
            if val is not None:
                arrays[f"obs{i}_{key}"] = val
    for k, v in ref.items():
        arrays[k] = np.asarray(v)
    arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(path, **arrays)


class Case:
    def __init__(self, path: str):
        z = np.load(path)
        self.path = path
        self.name = os.path.splitext(os.path.basename(path))[0]
        self.meta = json.loads(bytes(z["meta"]).decode())
        self.arrays = {k: z[k] for k in z.files if k != "meta"}
        self.spec = spec_from_meta(self.meta)

    def table_root(self) -> str:
        return syn.write_tables(self.spec, TABLE_ROOT)

    def star_root(self) -> str:
        """Directory holding this case's stellar spectrum file or grid ("" if none)."""
        kind = self.meta.get("star", "")
        if not kind:
            return ""
        return write_star(kind, self.arrays, os.path.join(TABLE_ROOT, "star_" + self.name) + "/")

    def config_text(self) -> str:
        return self.meta["config_template"].replace("{ROOT}", self.table_root()).replace("{STAR}", self.star_root())

    def observations(self) -> List[ObservationArrays]:
        out = []
        a = self.arrays
        for i, m in enumerate(self.meta["observations"]):
            g = lambda k: a.get(f"obs{i}_{k}")
            out.append(ObservationArrays(name=m["name"], type=m["type"], n=m["n"], centers_or_edges=g("ce"),
                                         data=g("data"), error=g("error"), weight=g("weight"), fwhm=g("fwhm"),
                                         filter_wavelength=g("fwl"), filter_response=g("fresp"),
                                         detector=m["detector"], modifier=m["modifier"]))
        return out

    @property
    def params(self) -> np.ndarray:
        return self.arrays["params"]

    def setup(self, k: int) -> dict:
        a = self.arrays
        return {"range": tuple(int(x) for x in a[f"ref_setup{k}_range"]),
                "edges": [tuple(int(x) for x in r) for r in a[f"ref_setup{k}_edges"]],
                "conv": [tuple(int(x) for x in r) for r in a[f"ref_setup{k}_conv"].reshape(-1, 2)]}


def write_star(kind: str, arrays: dict, folder: str) -> str:
    """Write a case's stellar spectrum ("file": folder/star.dat) or grid ("grid": the grid
    folder) from its arrays; returns the folder."""
    os.makedirs(folder, exist_ok=True)
    if kind == "file":
        syn.write_star_file(os.path.join(folder, "star.dat"), arrays["star_wl"], arrays["star_flux"])
    elif kind == "grid":
        axes = [arrays[f"star_axis{i}"] for i in range(3)]
        syn.write_star_grid(folder, axes, arrays["star_grid_wl"], arrays["star_grid_spectra"])
    else:
        raise ValueError(kind)
    return folder


# golden files that are not forward-model cases (the prior-transform table)
NOT_MODEL_CASES = {"priors.npz"}


def golden_cases() -> List[str]:
    return sorted(p for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz"))
                  if os.path.basename(p) not in NOT_MODEL_CASES)


def user_order_from_internal(obs: List[ObservationArrays], internal: np.ndarray) -> np.ndarray:
    """Reverse the observations the reference stores in descending-wavelength
    order back to the caller's order (ForwardModel::calcModel)."""
    out = np.empty_like(internal)
    off = 0
    for o in obs:
        n = o.n
        ce = o.centers_or_edges
        asc = n > 1 and ((ce.ndim == 1 and ce[0] < ce[1]) or (ce.ndim == 2 and ce[0, 0] < ce[-1, 0]))
        seg = internal[..., off:off + n]
        out[..., off:off + n] = seg[..., ::-1] if asc else seg
        off += n
    return out


def rel_err(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.maximum(np.abs(b), 1e-300)
    return float(np.max(np.abs(a - b) / den)) if a.size else 0.0
