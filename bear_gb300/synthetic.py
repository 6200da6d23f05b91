"""Seeded synthetic inputs in the reference's on-disk formats.

The reference ships no opacity database and no benchmark data set, so every
workload here is synthetic. Files follow the reference's loaders exactly:

* ``wavenumber_full.dat``: a count, then one wavenumber per entry
  (src/spectral_grid/spectral_grid.cpp:87-119).
* ``<folder>/filelist.dat``: first line ``"<mass> [log]"``, then
  ``"<p_bar> <T_K> <file>"`` rows (src/transport_coeff/opacity_species.cpp:66-122).
* each data file is raw float32 over the full global grid
  (src/transport_coeff/cross_section_file.cpp:33-68); with the ``log`` flag the
  values are log10 cross sections, which the loader exponentiates. Mass 0 means
  cm^2 (no conversion, src/transport_coeff/sampled_data.cpp:68-72).

The generated tables use the ``log`` storage and are built from MT19937
uniforms (Irwin-Hall sums) with basic IEEE arithmetic only, so a given seed
produces bit-identical files on x86-64 and aarch64.

Workload shapes (levels, grids, table sizes, observation sizes) are the ones of
the five benchmark configurations; see ``CONFIGS``.
"""

from __future__ import annotations

import dataclasses
import hashlib
import json
import os
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np

from .config import (Config, EmissionModelConfig, Observation, OccultationConfig, Prior,
                     TransmissionModelConfig)

PARSEC = 3.08567758135e18
R_JUPITER = 7.1492e9
R_SUN = 6.96342e10

LINE_SPECIES = ["H2O", "CO", "CH4", "CO2", "NH3", "HCN", "H2S", "C2H2", "TiO", "VO", "FeH", "SiO"]


@dataclass
class TableSpec:
    n_p: int
    p_min: float
    p_max: float
    n_t: int
    t_min: float
    t_max: float
    logsig_mean: float
    logsig_std: float


@dataclass
class WorkloadSpec:
    name: str
    model: str                      # "emission" | "transmission" | "joint"
    nu_min: float
    nu_max: float
    nu_step: float
    nb_levels: int
    p_bottom: float
    p_top: float
    species: List[str]
    table: TableSpec
    temperature: str                # "poly" | "const"
    cloud: bool
    batch: int
    seed: int
    obs_kind: str                   # which observation builder to use
    rayleigh: Tuple[str, ...] = ("H2",)


CONFIGS: Dict[str, WorkloadSpec] = {
    # 50 levels 100 -> 1e-3 bar, 4 line species on 10 log-p x 20 T, 1 cm^-1, 150-bin R=120 spectrum
    "emission_plain": WorkloadSpec(
        "emission_plain", "emission", 1500.0, 8500.0, 1.0, 50, 100.0, 1e-3,
        LINE_SPECIES[:4], TableSpec(10, 1e-3, 100.0, 20, 100.0, 3000.0, -22.0, 1.5),
        "poly", False, 1, 20261203, "emission_plain"),
    # 100 levels 10 -> 1e-6 bar, 8 species on 12 log-p x 25 T, 0.5 cm^-1, 300 transit-depth bins
    "transmission_plain": WorkloadSpec(
        "transmission_plain", "transmission", 2900.0, 20100.0, 0.5, 100, 10.0, 1e-6,
        LINE_SPECIES[:8], TableSpec(12, 1e-6, 10.0, 25, 200.0, 3500.0, -23.0, 2.0),
        "const", True, 1, 20261204, "transmission_plain", ("H2", "He")),
    # 512 live points, 80 levels, 6 species, 2000-12000 cm^-1, 120 + 40 + 8 bins
    "emission_batched": WorkloadSpec(
        "emission_batched", "emission", 1500.0, 12500.0, 1.0, 80, 100.0, 1e-3,
        LINE_SPECIES[:6], TableSpec(10, 1e-3, 100.0, 20, 100.0, 3000.0, -22.0, 1.5),
        "poly", False, 512, 20261205, "emission_batched"),
    # adjoint: the batched emission grid plus a grey cloud (fixed bottom), batch 256
    "emission_adjoint": WorkloadSpec(
        "emission_adjoint", "emission", 1500.0, 12500.0, 1.0, 80, 100.0, 1e-3,
        LINE_SPECIES[:6], TableSpec(10, 1e-3, 100.0, 20, 100.0, 3000.0, -22.0, 1.5),
        "poly", True, 256, 20261206, "emission_batched"),
    # joint emission + transmission, 150 levels, 12 species on 15 log-p x 30 T x 100001 nu
    "joint_large": WorkloadSpec(
        "joint_large", "joint", 1000.0, 26000.0, 0.25, 150, 100.0, 1e-6,
        LINE_SPECIES[:12], TableSpec(15, 1e-6, 100.0, 30, 100.0, 3500.0, -22.5, 1.75),
        "poly", True, 1024, 20261207, "joint_large", ("H2", "He")),
}


def scaled(spec: WorkloadSpec, **kw) -> WorkloadSpec:
    """A copy of ``spec`` with fields replaced (used for small test cases)."""
    return dataclasses.replace(spec, **kw)


# --------------------------------------------------------------------------- tables


def _boxcar5(x: np.ndarray) -> np.ndarray:
    """5-point running mean along the last axis, edge values repeated."""
    pad = np.concatenate([x[..., :1], x[..., :1], x, x[..., -1:], x[..., -1:]], axis=-1)
    c = np.cumsum(pad, axis=-1, dtype=np.float64)
    c = np.concatenate([np.zeros(c.shape[:-1] + (1,)), c], axis=-1)
    return (c[..., 5:] - c[..., :-5]) / 5.0


def _fmt(x: float) -> str:
    return repr(float(x))


def table_nodes(t: TableSpec) -> Tuple[np.ndarray, np.ndarray]:
    p = np.logspace(np.log10(t.p_min), np.log10(t.p_max), t.n_p)
    T = np.linspace(t.t_min, t.t_max, t.n_t)
    # round to short decimals so the text files hold the values exactly
    return np.array([float(f"{v:.6g}") for v in p]), np.array([float(f"{v:.6g}") for v in T])


def _spec_key(spec: WorkloadSpec) -> str:
    d = dataclasses.asdict(spec)
    d.pop("batch", None)
    d.pop("obs_kind", None)
    d["format"] = TABLE_FORMAT
    return hashlib.sha1(json.dumps(d, sort_keys=True).encode()).hexdigest()[:16]


TABLE_FORMAT = 2  # bump when the generated tables change


def write_tables(spec: WorkloadSpec, root: str) -> str:
    """Write the global wavenumber list and all opacity tables for ``spec``
    under ``root``; returns the directory (with trailing slash). Skips the work
    if a completed copy for the same spec already exists."""
    root = os.path.join(root, f"{spec.name}_{_spec_key(spec)}") + "/"
    done = os.path.join(root, ".complete")
    if os.path.exists(done):
        return root
    os.makedirs(root, exist_ok=True)
    rng = np.random.RandomState(spec.seed % (2**32))
    n_full = int(round((spec.nu_max - spec.nu_min) / spec.nu_step)) + 1
    nu = spec.nu_min + spec.nu_step * np.arange(n_full, dtype=np.float64)
    with open(os.path.join(root, "wavenumber_full.dat"), "w") as f:
        f.write(f"{n_full}\n")
        f.write("\n".join(_fmt(v) for v in nu))
        f.write("\n")

    p_nodes, t_nodes = table_nodes(spec.table)
    for s in spec.species:
        folder = os.path.join(root, s)
        os.makedirs(folder, exist_ok=True)
        shared = _normal_like(rng, n_full)
        rows = []
        with open(os.path.join(folder, "filelist.dat"), "w") as fl:
            # mass 0 (cm^2, no conversion); "log": the files hold log10 cross sections
            fl.write("0 log\n")
            for T in t_nodes:
                for p in p_nodes:
                    name = f"sigma_{p:.6g}_{T:.6g}.bin"
                    fl.write(f"{_fmt(p)} {_fmt(T)} {name}\n")
                    rows.append(name)
        for name in rows:
            own = _normal_like(rng, n_full)
            x = (0.7 * shared + 0.3 * own) * (1.0 / 0.7615773105863909)
            x = _boxcar5(x) * 2.23606797749979
            logsig = (spec.table.logsig_mean + spec.table.logsig_std * x).astype(np.float32)
            logsig.tofile(os.path.join(folder, name))

    # collision-induced absorption: one pressure row per temperature, smooth in T and nu
    # (log10 sigma = a + 0.2 (T/1000 - 1) - 0.434 ((nu - 4500) / 3500)^2 + ripple)
    for cia, amp in (("H2-H2", -46.0), ("H2-He", -46.5)):
        folder = os.path.join(root, "CIA", cia)
        os.makedirs(folder, exist_ok=True)
        with open(os.path.join(folder, "filelist.dat"), "w") as fl:
            fl.write("0 log\n")
            for T in t_nodes:
                name = f"cia_{T:.6g}.bin"
                fl.write(f"1 {_fmt(T)} {name}\n")
                u = (nu - 4500.0) / 3500.0
                v = (nu / 700.0 + T / 500.0) * 0.15915494309189535
                ripple = 0.1 * (v - np.floor(v) - 0.5) ** 2
                lg = amp + 0.2 * (T / 1000.0 - 1.0) - 0.4342944819032518 * u * u + ripple
                lg.astype(np.float32).tofile(os.path.join(folder, name))
    open(done, "w").close()
    return root


def _normal_like(rng: np.random.RandomState, n: int) -> np.ndarray:
    """Approximately standard-normal values from four MT19937 uniforms
    (Irwin-Hall). Uses only integer and basic IEEE arithmetic, so the tables are
    bit-identical on every platform."""
    s = rng.random_sample(n)
    for _ in range(3):
        s += rng.random_sample(n)
    return (s - 2.0) * 1.7320508075688772


# --------------------------------------------------------------------------- models


def _opacity_lists(spec: WorkloadSpec) -> Tuple[List[str], List[str]]:
    sym = list(spec.species) + ["CIA-H2-H2", "CIA-H2-He"]
    fold = list(spec.species) + ["CIA/H2-H2", "CIA/H2-He"]
    for r in spec.rayleigh:
        sym.append(r)
        fold.append("Rayleigh")
    return sym, fold


def model_config(spec: WorkloadSpec, kind: Optional[str] = None):
    kind = kind or spec.model
    sym, fold = _opacity_lists(spec)
    chem_models = ["iso", "bg"]
    chem_params = [list(spec.species), ["H2He"]]
    cloud = (["grey"], [["fb"]]) if spec.cloud else ([], [])
    if kind == "emission":
        temp = ("poly", ["5", "1"]) if spec.temperature == "poly" else ("const", [])
        return EmissionModelConfig(spec.nb_levels, spec.p_bottom, spec.p_top, temp[0], temp[1],
                                   "scm", [], chem_models, chem_params, sym, fold,
                                   cloud[0], cloud[1])
    temp = ("const", []) if (spec.temperature == "const" or spec.model == "joint") else ("poly", ["5", "1"])
    if spec.model == "joint":
        temp = ("poly", ["5", "1"])
    return TransmissionModelConfig(False, False, False, spec.nb_levels, spec.p_bottom, spec.p_top,
                                   temp[0], temp[1], chem_models, chem_params, sym, fold,
                                   cloud[0], cloud[1], [], [])


def global_config(spec: WorkloadSpec, table_root: str, kind: Optional[str] = None) -> Config:
    cfg = Config(True, kind or spec.model, table_root, "const_wavenumber", spec.nu_step, "", "")
    cfg.wavenumber_file_path = table_root + "wavenumber_full.dat"
    return cfg


def priors(spec: WorkloadSpec, kind: Optional[str] = None) -> List[Prior]:
    """Priors of each workload. Batched live points are drawn uniformly over
    these (cube ~ U[0,1]^P mapped through each prior)."""
    kind = kind or spec.model
    pr: List[Prior] = []
    if kind == "emission":
        pr.append(Prior("uniform", "log g", [4.5, 5.5]))
        pr.append(Prior("uniform", "scaling f", [0.5, 2.0]))
        pr.append(Prior("delta", "distance", [10.0], "pc"))
    else:
        pr.append(Prior("delta", "log g", [3.0]))
        pr.append(Prior("delta", "R_p", [1.2], "Rj"))
        pr.append(Prior("delta", "R_s", [1.0], "Rs"))
    lo, hi = (1e-8, 1e-3) if kind == "emission" else (1e-10, 1e-2)
    for s in spec.species:
        pr.append(Prior("log_uniform", s, [lo, hi]))
    if kind == "emission" or spec.model == "joint":
        if spec.temperature == "poly" or spec.model == "joint":
            pr.append(Prior("uniform", "T0", [1000.0, 3000.0]))
            for k in range(5):
                pr.append(Prior("uniform", f"T ratio {k+1}", [0.6, 1.0]))
        else:
            pr.append(Prior("uniform", "T", [800.0, 2500.0]))
    else:
        pr.append(Prior("uniform", "T", [800.0, 2500.0]))
    if spec.cloud:
        pr.append(Prior("delta" if kind == "transmission" else "log_uniform",
                        "cloud optical depth", [10.0] if kind == "transmission" else [0.1, 10.0]))
        p_lo = max(spec.p_top * 10.0, 1e-5)
        p_hi = min(spec.p_bottom / 10.0, 10.0)
        pr.append(Prior("log_uniform", "cloud top pressure", [p_lo, p_hi]))
    return pr


_UNITS = {"": 1.0, "pc": PARSEC, "Rj": R_JUPITER, "Rs": R_SUN}


def cube_to_physical(pr: Sequence[Prior], cube: np.ndarray) -> np.ndarray:
    """Map hypercube points to physical parameters the way the reference's
    uniform / log-uniform / delta priors do (src/retrieval/prior_types.h:89-230,
    unit factors :57-82)."""
    cube = np.atleast_2d(np.asarray(cube, dtype=np.float64))
    out = np.empty_like(cube)
    for j, p in enumerate(pr):
        u = _UNITS[p.unit]
        if p.type == "uniform":
            lo, hi = sorted(p.parameter)
            out[:, j] = (lo + cube[:, j] * (hi - lo)) * u
        elif p.type == "log_uniform":
            lo, hi = sorted(np.log10(p.parameter))
            out[:, j] = np.power(10.0, lo + cube[:, j] * (hi - lo)) * u
        elif p.type == "delta":
            out[:, j] = p.parameter[0] * u
        else:
            raise ValueError(f"prior type {p.type} not supported here")
    return out


def truth_parameters(spec: WorkloadSpec, kind: Optional[str] = None, index: int = 0) -> np.ndarray:
    """One seeded physical parameter set (seed = workload seed + 1000 * index)."""
    kind = kind or spec.model
    rng = np.random.default_rng(spec.seed + 1000 * index + (17 if kind == "transmission" else 0))
    pr = priors(spec, kind)
    if spec.name == "emission_plain" and kind == "emission" and index == 0:
        # the plain emission case: log g 5, f 1, 10 pc, knots U[300,2500], log x U[-8,-3]
        x = 10.0 ** rng.uniform(-8, -3, len(spec.species))
        knots = rng.uniform(300.0, 2500.0, 6)
        ratios = knots[1:] / knots[:-1]
        return np.concatenate([[5.0, 1.0, 10.0 * PARSEC], x, [knots[0]], ratios])
    return cube_to_physical(pr, rng.uniform(0.0, 1.0, (1, len(pr))))[0]


# --------------------------------------------------------------------------- observations


def _gauss_filter(nu_c: float, width: float) -> Tuple[np.ndarray, np.ndarray]:
    nu = np.linspace(nu_c - width, nu_c + width, 61)
    resp = np.exp(-0.5 * ((nu - nu_c) / (width / 2.355)) ** 2)
    return 1e4 / nu, resp


def _tophat_filter(nu_c: float, width: float) -> Tuple[np.ndarray, np.ndarray]:
    nu = np.linspace(nu_c - 0.5 * width - 2.0, nu_c + 0.5 * width + 2.0, 41)
    resp = np.where(np.abs(nu - nu_c) <= 0.5 * width, 1.0, 0.0)
    return 1e4 / nu, resp


def observations(spec: WorkloadSpec, kind: Optional[str] = None) -> List[Observation]:
    """Observation layouts with placeholder data (ones); ``attach_data`` fills
    data and errors from a model evaluation."""
    kind = kind or spec.model
    rng = np.random.default_rng(spec.seed + 7)
    obs: List[Observation] = []
    k = spec.obs_kind
    if k == "emission_plain":
        wl = np.linspace(1.25, 5.0, 150)
        o = Observation("spex_like", "spectroscopy", wl, np.ones(150), np.ones(150))
        o.instrument_profile_fwhm = list(wl / 120.0)
        obs.append(o)
    elif k == "transmission_plain":
        edges = np.geomspace(0.5003, 3.332, 301)
        bins = np.stack([edges[:-1], edges[1:]], axis=1)
        obs.append(Observation("transit_bins", "band-spectroscopy", bins, np.ones(300), np.ones(300)))
    elif k == "emission_batched":
        wl = np.linspace(0.85, 4.85, 120)
        o = Observation("prism_like", "spectroscopy", wl, np.ones(120), np.ones(120))
        o.instrument_profile_fwhm = list(wl / 100.0)
        obs.append(o)
        edges = np.linspace(1.1, 1.7, 41)
        bins = np.stack([edges[:-1], edges[1:]], axis=1)
        obs.append(Observation("wfc3_like", "band-spectroscopy", bins, np.ones(40), np.ones(40)))
        centres = np.geomspace(2300.0, 9500.0, 8)
        widths = np.linspace(50.0, 400.0, 8)
        for i, (c, w) in enumerate(zip(centres, widths)):
            fw, fr = (_tophat_filter if i % 2 == 0 else _gauss_filter)(c, w)
            edge = [1e4 / (c - 0.5 * w), 1e4 / (c + 0.5 * w)]
            o = Observation(f"phot_{i}", "photometry", [edge], np.ones(1), np.ones(1))
            o.filter_response = [list(fw), list(fr)]
            o.filter_detector_type = "energy" if i % 3 else "photon"
            obs.append(o)
    elif k == "joint_large":
        if kind == "emission":
            layout = [("em_vis", 0.405, 2.5, 300, "spectroscopy"), ("em_ir", 2.5, 9.5, 150, "spectroscopy")]
        else:
            layout = [("tr_vis", 0.4, 3.0, 300, "spectroscopy"), ("tr_ir", 3.0, 9.5, 150, "band-spectroscopy")]
        for name, a, b, n, typ in layout:
            if typ == "spectroscopy":
                wl = np.geomspace(a, b, n)
                o = Observation(name, typ, wl, np.ones(n), np.ones(n))
                centres = wl
            else:
                edges = np.geomspace(a, b, n + 1)
                bins = np.stack([edges[:-1], edges[1:]], axis=1)
                o = Observation(name, typ, bins, np.ones(n), np.ones(n))
                centres = np.sqrt(edges[:-1] * edges[1:])
            # resolving power varying per bin between 100 and 3000
            R = np.exp(np.linspace(np.log(3000.0), np.log(100.0), n))
            o.instrument_profile_fwhm = list(centres / R)
            obs.append(o)
    else:
        raise ValueError(k)
    return obs


def attach_data(obs: List[Observation], model_obs: Sequence[np.ndarray], kind: str, seed: int) -> None:
    """data = model (1 + 1% N(0,1)) with 1% errors for emission fluxes;
    data = model + N(0, 50 ppm) with 50 ppm errors for transit depths."""
    rng = np.random.default_rng(seed + 99)
    for o, m in zip(obs, model_obs):
        m = np.asarray(m, dtype=np.float64)
        if kind == "emission":
            err = 0.01 * np.abs(m)
            err[err == 0] = 1e-30
            data = m * (1.0 + 0.01 * rng.standard_normal(m.shape))
        else:
            err = np.full(m.shape, 50.0)
            data = m + 50.0 * rng.standard_normal(m.shape)
        o.data = list(data)
        o.data_error = list(err)


# --------------------------------------------------------------------------- secondary eclipse
# Stellar spectra for the secondary-eclipse model: surface flux in W m^-2 um^-1 (the
# reference's stellar file unit), pi B_lambda(T_eff) with seeded absorption lines whose
# depth grows with [M/H] and whose width grows with log g.

_H, _C, _K = 6.62606896e-34, 2.99792458e8, 1.3806504e-23   # SI


def star_spectrum(teff: float, log_g: float = 4.5, metallicity: float = 0.0, n: int = 3000,
                  wl_min: float = 0.3, wl_max: float = 30.0, seed: int = 5) -> Tuple[np.ndarray, np.ndarray]:
    """(wavelengths in um ascending, flux in W m^-2 um^-1) of a synthetic star."""
    wl = np.geomspace(wl_min, wl_max, n)
    lam = wl * 1e-6
    b_lambda = 2.0 * _H * _C**2 / lam**5 / np.expm1(_H * _C / (lam * _K * teff)) * 1e-6
    rng = np.random.default_rng(seed)
    centres = np.geomspace(wl_min, wl_max, 60) * np.exp(rng.uniform(-0.02, 0.02, 60))
    depth = rng.uniform(0.05, 0.3, 60) * (1.0 + 0.5 * metallicity)
    width = rng.uniform(0.002, 0.01, 60) * (1.0 + 0.2 * (log_g - 4.5))
    lines = np.ones_like(wl)
    for c, d, w in zip(centres, depth, width):
        lines *= 1.0 - d * np.exp(-0.5 * ((np.log(wl) - np.log(c)) / w) ** 2)
    return wl, np.pi * b_lambda * lines


def write_star_file(path: str, wl: np.ndarray, flux: np.ndarray) -> None:
    """Stellar spectrum file of the "file" model: one "wavelength flux" line per point."""
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        for a, b in zip(wl, flux):
            f.write(f"{_fmt(a)} {_fmt(b)}\n")
    os.replace(tmp, path)


def star_grid(teff: Sequence[float], log_g: Sequence[float], metallicity: Sequence[float],
              n: int = 2000) -> Tuple[List[np.ndarray], np.ndarray, np.ndarray]:
    """Axes, float32 wavelengths and float32 spectra (T_eff, log g, [M/H] row-major) of a
    synthetic stellar grid."""
    axes = [np.asarray(teff, dtype=np.float64), np.asarray(log_g, dtype=np.float64),
            np.asarray(metallicity, dtype=np.float64)]
    spectra = []
    for t in axes[0]:
        for g in axes[1]:
            for m in axes[2]:
                wl, fl = star_spectrum(float(t), float(g), float(m), n=n)
                spectra.append(fl)
    return axes, wl.astype(np.float32), np.asarray(spectra, dtype=np.float32)


def write_star_grid(folder: str, axes: Sequence[np.ndarray], wl: np.ndarray, spectra: np.ndarray) -> None:
    """Stellar grid folder of the "grid" model: grid_parameters.dat (three node lines, the
    wavelength file name, then "T_eff log_g [M/H] file" per spectrum) and float32 files."""
    os.makedirs(folder, exist_ok=True)
    np.asarray(wl, dtype=np.float32).tofile(os.path.join(folder, "wavelengths.bin"))
    lines = [" ".join(_fmt(v) for v in a) for a in axes] + ["wavelengths.bin"]
    i = 0
    for t in axes[0]:
        for g in axes[1]:
            for m in axes[2]:
                name = f"spectrum_{i:03d}.bin"
                np.asarray(spectra[i], dtype=np.float32).tofile(os.path.join(folder, name))
                lines.append(f"{_fmt(t)} {_fmt(g)} {_fmt(m)} {name}")
                i += 1
    tmp = os.path.join(folder, "grid_parameters.dat.tmp")
    with open(tmp, "w") as f:
        f.write("\n".join(lines) + "\n")
    os.replace(tmp, os.path.join(folder, "grid_parameters.dat"))


def eclipse_model_config(spec: WorkloadSpec, star_model: str, star_params: Sequence[str]) -> OccultationConfig:
    """The emission workload's atmosphere as a secondary-eclipse model."""
    sym, fold = _opacity_lists(spec)
    temp = ("poly", ["5", "1"]) if spec.temperature == "poly" else ("const", [])
    cloud = (["grey"], [["fb"]]) if spec.cloud else ([], [])
    return OccultationConfig(spec.nb_levels, spec.p_bottom, spec.p_top, temp[0], temp[1], "scm", [],
                             ["iso", "bg"], [list(spec.species), ["H2He"]], sym, fold, star_model,
                             list(star_params), cloud[0], cloud[1])


def eclipse_priors(spec: WorkloadSpec, star_model: str, axes: Optional[Sequence[np.ndarray]] = None) -> List[Prior]:
    """[log g, R_p / R_s, stellar parameters, abundances, temperature, cloud] of an eclipse workload."""
    pr = [Prior("uniform", "log g", [3.0, 3.6]), Prior("uniform", "R_p/R_s", [0.08, 0.14])]
    if star_model == "blackbody":
        pr.append(Prior("uniform", "T_eff", [4500.0, 6500.0]))
    elif star_model == "grid":
        for name, a in zip(("T_eff", "stellar log g", "[M/H]"), axes):
            pr.append(Prior("uniform", name, [float(a[0]), float(a[-1])]))
    for sp in spec.species:
        pr.append(Prior("log_uniform", sp, [1e-8, 1e-3]))
    if spec.temperature == "poly":
        pr.append(Prior("uniform", "T0", [1200.0, 2800.0]))
        for k in range(5):
            pr.append(Prior("uniform", f"T ratio {k+1}", [0.6, 1.0]))
    else:
        pr.append(Prior("uniform", "T", [900.0, 2500.0]))
    if spec.cloud:
        pr.append(Prior("log_uniform", "cloud optical depth", [0.1, 10.0]))
        pr.append(Prior("log_uniform", "cloud top pressure", [max(spec.p_top * 10.0, 1e-5),
                                                              min(spec.p_bottom / 10.0, 10.0)]))
    return pr
