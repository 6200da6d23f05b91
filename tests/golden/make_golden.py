"""Generates the golden cases under tests/golden/ by running the reference's own
CPU path (oracle/_ref/bear_ref_harness, built from the reference sources by
oracle/ref/Makefile) on seeded synthetic inputs.

    make -C oracle/ref REF=<reference sources> && python tests/golden/make_golden.py [case ...]

The prior-transform case (tests/golden/priors.npz) is made with the argument "priors".

Each case: tables from bear_gb300.synthetic (regenerated at test time), a
config-text template, observations whose data are the reference model at a
seeded parameter set plus seeded noise, and the reference's outputs for a few
parameter sets. See tests/goldenlib.py for the file layout.
"""

from __future__ import annotations

import dataclasses
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.dirname(HERE))

import refcase  # noqa: E402
from bear_gb300 import synthetic as syn  # noqa: E402
from bear_gb300.config import Observation, observation_arrays, render_config  # noqa: E402
from goldenlib import GOLDEN_DIR, TABLE_ROOT, save_case, spec_to_meta, write_star  # noqa: E402


def run_ref(name, template, root, obs, params, star_dir=""):
    d = os.path.join("/tmp", "bear_golden_case_" + name)
    refcase.write_case(d, template.replace("{ROOT}", root).replace("{STAR}", star_dir),
                       [observation_arrays(o) for o in obs], params)
    return refcase.run_case(d)


def split_obs(obs, flat):
    out, off = [], 0
    for o in obs:
        out.append(flat[off:off + len(o.data)])
        off += len(o.data)
    return out


def make(name, spec, kind, template_fn, obs, params, spectrum_rows, attach_kind=None, truth_index=0,
         model_cfg=None, star=None):
    """star: (kind, arrays) of a secondary-eclipse case's stellar file or grid."""
    root = syn.write_tables(spec, TABLE_ROOT)
    mc = model_cfg if model_cfg is not None else syn.model_config(spec, kind)
    template = template_fn(render_config(syn.global_config(spec, "{ROOT}", kind), mc))
    star_dir = write_star(star[0], star[1], os.path.join(TABLE_ROOT, "star_" + name) + "/") if star else ""
    # data: the reference model at the truth parameters plus seeded noise
    first = run_ref(name, template, root, obs, params[truth_index:truth_index + 1], star_dir)
    syn.attach_data(obs, split_obs(obs, first["obs"][0]), attach_kind or kind, spec.seed)
    ref = run_ref(name, template, root, obs, params, star_dir)
    arrays = [observation_arrays(o) for o in obs]
    out = {
        "ref_loglike": ref["loglike"], "ref_neglect": ref["neglect"], "ref_obs": ref["obs"],
        "ref_grid": ref["grid"], "spectrum_rows": np.array(spectrum_rows, dtype=np.int64),
        "ref_spectrum": ref["spectrum"][spectrum_rows],
    }
    for k, s in enumerate(ref["setup"]):
        out[f"ref_setup{k}_range"] = np.array(s["range"], dtype=np.int64)
        out[f"ref_setup{k}_edges"] = np.array(s["edges"], dtype=np.int64).reshape(-1, 2)
        out[f"ref_setup{k}_conv"] = np.array(s["conv"], dtype=np.int64).reshape(-1, 2)
    meta = {"spec": spec_to_meta(spec), "kind": kind, "config_template": template}
    if star:
        meta["star"] = star[0]
        out.update(star[1])
    save_case(os.path.join(GOLDEN_DIR, name + ".npz"), meta, arrays, params, out)
    print(f"{name}: N={ref['grid'].size} M={ref['obs'].shape[1]} S={params.shape[0]} loglike={ref['loglike']}")


def same(t):
    return t


# prior list of the prior-transform case: one per parameter of the emission edge-case model
# (log g, f, distance, H2O, CO, K, T, cloud tau, cloud top, bottom factor, shift, error
# exponent), every type but the Gaussian (the reference's erf_inv comes from Boost.Math,
# which is not in the image) and every unit; linked priors give the 1-based index they follow
PRIOR_CASE = [
    ("uniform", "log_g", [5.5, 4.5], ""),            # reversed bounds: swapped by the reference
    ("log_uniform", "scaling_f", [0.5, 2.0], "Rs"),
    ("delta", "distance", [10.0], "pc"),
    ("log_uniform", "H2O", [1e-8, 1e-2], ""),
    ("linked", "CO", [4.0], ""),                     # follows H2O's cube coordinate
    ("log_uniform", "K", [1e-5, 1e-9], "Me"),        # reversed bounds
    ("uniform", "T", [800.0, 2500.0], "Rj"),
    ("uniform", "cloud_tau", [0.0, 10.0], "Mj"),
    ("log_uniform", "cloud_top", [1e-3, 1.0], "Ms"),
    ("linked", "bottom_factor", [7.0], ""),          # follows T's cube coordinate, without T's unit
    ("uniform", "shift", [-1e-3, 1e-3], "ly"),
    ("uniform", "error_exponent", [-40.0, -30.0], "Re"),
]


def make_priors():
    """Retrieval::convertCubeParameters of the reference on seeded hypercube points (and the
    corners 0, 1, 1/2) with PRIOR_CASE on the emission edge-case model."""
    import json

    from bear_gb300.config import Prior
    from goldenlib import Case

    base = Case(os.path.join(GOLDEN_DIR, "emission_edges.npz"))
    pr = [Prior(t, d, list(p), u) for t, d, p, u in PRIOR_CASE]
    P = len(pr)
    cube = np.random.default_rng(20261212).uniform(size=(61, P))
    cube = np.vstack([np.zeros(P), np.ones(P), np.full(P, 0.5), cube])
    ref = refcase.run_priors(os.path.join("/tmp", "bear_golden_case_priors"), base.config_text(),
                             base.observations(), pr, cube)
    meta = {"base_case": "emission_edges", "priors": [list(x) for x in PRIOR_CASE]}
    np.savez_compressed(os.path.join(GOLDEN_DIR, "priors.npz"), cube=cube, ref_parameter=ref["parameter"],
                        ref_physical=ref["physical"],
                        meta=np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8))


def main():
    os.makedirs(GOLDEN_DIR, exist_ok=True)
    which = set(sys.argv[1:])

    # prior transforms of the reference (the emission edge-case model must exist already)
    if "priors" in which:
        make_priors()
        return

    # 1. plain emission, the 50-level / 6270-point benchmark workload
    if not which or "emission_plain" in which:
        spec = syn.CONFIGS["emission_plain"]
        obs = syn.observations(spec, "emission")
        params = np.stack([syn.truth_parameters(spec, "emission", i) for i in range(3)])
        make("emission_plain", spec, "emission", same, obs, params, [0, 1, 2])

    # 2. plain transmission, 100 levels / 34k points, grey cloud, H2 + He Rayleigh
    if not which or "transmission_plain" in which:
        spec = syn.CONFIGS["transmission_plain"]
        obs = syn.observations(spec, "transmission")
        params = np.stack([syn.truth_parameters(spec, "transmission", i) for i in range(3)])
        make("transmission_plain", spec, "transmission", same, obs, params, [0])

    # 3. three observation kinds of the batched workload: R=100 spectrum, bins, 8 filters
    if not which or "emission_batched" in which:
        spec = syn.CONFIGS["emission_batched"]
        obs = syn.observations(spec, "emission")
        params = np.stack([syn.truth_parameters(spec, "emission", i) for i in range(4)])
        make("emission_batched", spec, "emission", same, obs, params, [0])

    # 4. emission edge cases: 2 cm^-1 sampling, const T on a table node, grey cloud with
    #    bottom fraction, K (sodium follows potassium), shift modifier, error inflation,
    #    ascending / descending / photon-counting observations, a neglected point
    if not which or "emission_edges" in which:
        spec = dataclasses.replace(syn.CONFIGS["emission_plain"], name="emission_edges", nb_levels=40,
                                   species=["H2O", "CO", "K", "Na"], temperature="const", seed=20261210)
        spec = dataclasses.replace(spec, obs_kind="emission_plain")

        def tmpl(t):
            t = t.replace("spectral_resolution 1.0", "spectral_resolution 2.0")
            t = t.replace("error_inflation 0", "error_inflation 1")
            t = t.replace("temperature_profile poly 5 1", "temperature_profile const")
            t = t.replace("chemistry iso H2O CO K Na", "chemistry iso H2O CO K")
            return t + "cloud grey\n"
        wl = np.linspace(1.4, 4.6, 60)
        o1 = Observation("asc_spec", "spectroscopy", wl, np.ones(60), np.ones(60))
        o1.instrument_profile_fwhm = list(wl / 150.0)
        o1.likelihood_weight = list(np.linspace(0.5, 1.5, 60))
        o1.spectrum_modifier_id = "shift_const"
        edges = np.linspace(4.0, 2.2, 21)
        bins = np.stack([edges[:-1], edges[1:]], axis=1)
        o2 = Observation("desc_bins", "band-spectroscopy", bins, np.ones(20), np.ones(20))
        fw = np.linspace(2.05, 2.45, 30)
        o3 = Observation("photon_filter", "photometry", [[2.45, 2.05]], np.ones(1), np.ones(1))
        o3.filter_response = [list(fw), list(np.exp(-0.5 * ((fw - 2.25) / 0.08) ** 2))]
        o3.filter_detector_type = "Photon"
        obs = [o1, o2, o3]
        base = [5.0, 1.0, 10 * syn.PARSEC, 3e-4, 1e-4, 2e-7]   # log g, f, d, H2O, CO, K
        T_node = float(syn.table_nodes(spec.table)[1][8])       # exactly a table temperature
        rows = []
        for T, cloud, shift in ((1500.0, [3.0, 0.05, 5.0], 0.0), (T_node, [1.0, 0.3, 3.0], 1e-16),
                                (2200.0, [0.0, 0.01, 10.0], -2e-16)):
            rows.append(base + [T] + cloud + [shift, -36.0])
        bad = list(rows[0])
        bad[3] = 0.7  # mixing ratios sum above one: neglected, log L = -1e30
        bad[4] = 0.5
        rows.append(bad)
        make("emission_edges", spec, "emission", tmpl, obs, np.array(rows), [0, 1])

    # 5. transmission edge cases: variable gravity, fitted mean molecular weight, poly T,
    #    ascending bins with an instrument profile, an energy-counting filter, inflation
    if not which or "transmission_edges" in which:
        spec = dataclasses.replace(syn.CONFIGS["transmission_plain"], name="transmission_edges", nb_levels=60,
                                   nu_min=2900.0, nu_max=12100.0, species=["H2O", "CH4", "CO2"],
                                   temperature="poly", seed=20261211)

        def tmpl(t):
            t = t.replace("error_inflation 0", "error_inflation 1")
            t = t.replace("temperature_profile poly 5 1", "temperature_profile poly 3 1")
            assert "temperature_profile poly 3 1" in t
            t = t.replace("fit_mean_molecular_weight 0", "fit_mean_molecular_weight 1")
            t = t.replace("variable_gravity 0", "variable_gravity 1")
            return t
        edges = np.geomspace(0.9, 3.3, 41)
        bins = np.stack([edges[:-1], edges[1:]], axis=1)
        o1 = Observation("asc_bins", "band-spectroscopy", bins, np.ones(40), np.ones(40))
        o1.instrument_profile_fwhm = list(np.sqrt(edges[:-1] * edges[1:]) / 200.0)
        fw = np.linspace(1.1, 1.6, 40)
        o2 = Observation("energy_filter", "photometry", [[1.1, 1.6]], np.ones(1), np.ones(1))
        o2.filter_response = [list(fw), list(np.where((fw > 1.2) & (fw < 1.5), 1.0, 0.05))]
        o2.filter_detector_type = "energy"
        obs = [o1, o2]
        rows = []
        for logg, mmw, T, cl in ((3.0, 2.3, [1400.0, 0.9, 0.95, 0.8], [10.0, 1e-3]),
                                 (3.3, 2.5, [900.0, 1.1, 0.9, 1.0], [10.0, 1e-2]),
                                 (2.8, 2.2, [2000.0, 0.8, 0.8, 0.9], [10.0, 3e-4])):
            rows.append([logg, 1.2 * syn.R_JUPITER, syn.R_SUN, mmw, 1e-4, 1e-5, 1e-6] + T + cl + [2.0])
        cold = list(rows[0])
        cold[7] = 60.0   # the profile drops below 50 K: neglected
        rows.append(cold)
        make("transmission_edges", spec, "transmission", tmpl, obs, np.array(rows), [0, 1],
             attach_kind="transmission")

    # 9. transmission with every Rayleigh species of the reference (H2, He, H, CO, CO2, CH4,
    #    H2O; the last four vanish beyond 2 micron), atomic H in the chemistry, 0.45-3.4 um
    if not which or "transmission_rayleigh" in which:
        spec = dataclasses.replace(syn.CONFIGS["transmission_plain"], name="transmission_rayleigh", nb_levels=50,
                                   nu_min=2900.0, nu_max=22500.0, nu_step=2.0, species=["H2O", "CO", "CO2", "CH4"],
                                   temperature="const", cloud=False, seed=20261230,
                                   rayleigh=("H2", "He", "H", "CO", "CO2", "CH4", "H2O"))

        def tmpl(t):
            assert "chemistry iso H2O CO CO2 CH4\n" in t
            return t.replace("chemistry iso H2O CO CO2 CH4\n", "chemistry iso H2O CO CO2 CH4 H\n")
        edges = np.geomspace(0.46, 3.3, 61)
        obs = [Observation("transit_bins", "band-spectroscopy", np.stack([edges[:-1], edges[1:]], axis=1),
                           np.ones(60), np.ones(60))]
        rows = []
        for T, xs, xh in ((1200.0, [1e-4, 1e-4, 1e-6, 1e-5], 1e-3), (800.0, [1e-3, 1e-5, 1e-7, 1e-4], 1e-5),
                          (2200.0, [1e-6, 1e-3, 1e-5, 1e-8], 0.05)):
            rows.append([3.2, 1.1 * syn.R_JUPITER, 0.9 * syn.R_SUN] + xs + [xh, T])
        make("transmission_rayleigh", spec, "transmission", tmpl, obs, np.array(rows), [0, 2],
             attach_kind="transmission")

    # 10-11. the H- bound-free + free-free continuum (GasHm) with H, H- and e- in the chemistry,
    #        in a hot emission model and a transmission model, 0.33-3.3 um
    for kind in ("emission", "transmission"):
        name = f"{kind}_hminus"
        if which and name not in which:
            continue
        base = syn.CONFIGS["emission_plain" if kind == "emission" else "transmission_plain"]
        spec = dataclasses.replace(base, name=name, model=kind, nb_levels=45, nu_min=3000.0, nu_max=30500.0,
                                   nu_step=4.0, species=["H2O", "CO"],
                                   temperature="poly" if kind == "emission" else "const", cloud=False,
                                   seed=20261240 + (kind == "transmission"),
                                   rayleigh=() if kind == "emission" else ("H2",))

        def tmpl(t):
            assert "chemistry iso H2O CO\n" in t
            t = t.replace("chemistry iso H2O CO\n", "chemistry iso H2O CO H H- e-\n")
            return t + "opacity H-\n"
        edges = np.geomspace(0.34, 3.2, 51)
        o1 = Observation("bins", "band-spectroscopy", np.stack([edges[:-1], edges[1:]], axis=1), np.ones(50),
                         np.ones(50))
        wl = np.geomspace(0.5, 1.6, 30)
        o2 = Observation("spec", "spectroscopy", wl, np.ones(30), np.ones(30))
        o2.instrument_profile_fwhm = list(wl / 300.0)
        obs = [o1, o2]
        rows = []
        for T, xs in ((2600.0, [1e-4, 3e-4, 1e-3, 3e-9, 1e-6]), (3400.0, [1e-5, 1e-4, 1e-2, 1e-8, 1e-5]),
                      (1900.0, [1e-3, 1e-3, 1e-5, 1e-10, 1e-8])):
            if kind == "emission":  # an inverted-free profile falling from T to 0.55 T at the top
                rows.append([4.5, 1.0, 10 * syn.PARSEC] + xs + [T, 0.95, 0.9, 0.85, 0.8, 0.85])
            else:
                rows.append([3.0, 1.4 * syn.R_JUPITER, syn.R_SUN] + xs + [T])
        zero = list(rows[0])
        zero[6] = 0.0   # no H-: the reference skips the whole continuum (free-free included)
        rows.append(zero)
        make(name, spec, kind, tmpl, obs, np.array(rows), [0, 1], attach_kind=kind)

    # 12-13. non-grey clouds: a power-law cloud (reference wavelength 1 um, free bottom) in
    #        emission and a KH non-grey cloud (reference 1.5 um, fixed bottom) in transmission
    for name, kind, cl in (("emission_powerlaw_cloud", "emission", "cloud power_law 1.0\n"),
                           ("transmission_kh_cloud", "transmission", "cloud KHnongrey 1.5 fb\n")):
        if which and name not in which:
            continue
        base = syn.CONFIGS["emission_plain" if kind == "emission" else "transmission_plain"]
        spec = dataclasses.replace(base, name=name, model=kind, nb_levels=50, nu_min=2500.0, nu_max=16500.0,
                                   nu_step=2.0, species=["H2O", "CO", "CH4"], cloud=False, seed=20261250 + len(kind),
                                   temperature="poly" if kind == "emission" else "const")

        def tmpl(t, cl=cl):
            return t + cl
        edges = np.geomspace(0.65, 3.8, 49)
        o1 = Observation("bins", "band-spectroscopy", np.stack([edges[:-1], edges[1:]], axis=1), np.ones(48),
                         np.ones(48))
        wl = np.geomspace(1.0, 2.5, 40)
        o2 = Observation("spec", "spectroscopy", wl, np.ones(40), np.ones(40))
        o2.instrument_profile_fwhm = list(wl / 200.0)
        obs = [o1, o2]
        rows = []
        if kind == "emission":
            for tau, a, ptop, frac, T in ((2.0, -2.0, 0.3, 8.0, 1600.0), (8.0, -4.0, 1.0, 3.0, 2100.0),
                                          (0.5, 1.0, 0.05, 20.0, 1200.0)):
                rows.append([4.8, 1.0, 10 * syn.PARSEC, 1e-4, 3e-4, 1e-6, T, 0.9, 0.85, 0.8, 0.85, 0.9,
                             tau, a, ptop, frac])
        else:
            for tau, q0, a0, r, ptop, T in ((5.0, 10.0, 4.0, 0.5, 0.01, 1300.0), (20.0, 3.0, 6.0, 1.5, 1e-3, 900.0),
                                            (1.0, 30.0, 2.0, 0.1, 0.1, 1900.0)):
                rows.append([3.1, 1.3 * syn.R_JUPITER, syn.R_SUN, 1e-4, 1e-4, 1e-5, T, tau, q0, a0, r, ptop])
        make(name, spec, kind, tmpl, obs, np.array(rows), [0, 1], attach_kind=kind)

    # 6-8. secondary eclipse (occultation depth, ppm) with a blackbody, a file and a grid star:
    #      40 levels, 2 cm^-1 sampling from 1.0 to 6.7 um, an R=100 spectrum with an instrument
    #      profile and a shift modifier, descending bins, two photon-counting filters
    for star_kind in ("blackbody", "file", "grid"):
        name = "eclipse_" + star_kind
        if which and name not in which:
            continue
        spec = dataclasses.replace(syn.CONFIGS["emission_plain"], name=name, model="emission", nb_levels=40,
                                   nu_min=1500.0, nu_max=10000.0, nu_step=2.0, species=["H2O", "CO", "CH4"],
                                   temperature="poly", cloud=(star_kind == "file"), seed=20261220)
        star = None
        star_params = []
        axes = None
        if star_kind == "file":
            wl, fl = syn.star_spectrum(5200.0, 4.4, 0.1)
            star = ("file", {"star_wl": wl[::-1].copy(), "star_flux": fl[::-1].copy()})  # descending file
            star_params = ["{STAR}star.dat"]
        elif star_kind == "grid":
            axes, gwl, gsp = syn.star_grid([4000.0, 4600.0, 5300.0, 6000.0], [4.0, 4.5], [-0.5, 0.0, 0.5])
            star = ("grid", {"star_axis0": axes[0], "star_axis1": axes[1], "star_axis2": axes[2],
                             "star_grid_wl": gwl, "star_grid_spectra": gsp})
            star_params = ["{STAR}"]
        mc = syn.eclipse_model_config(spec, star_kind, star_params)
        wl = np.geomspace(1.1, 5.0, 40)
        o1 = Observation("nirspec_like", "spectroscopy", wl, np.ones(40), np.ones(40))
        o1.instrument_profile_fwhm = list(wl / 100.0)
        o1.spectrum_modifier_id = "shift_const"
        edges = np.linspace(1.7, 1.1, 13)
        o2 = Observation("wfc3_bins", "band-spectroscopy", np.stack([edges[:-1], edges[1:]], axis=1),
                         np.ones(12), np.ones(12))
        obs = [o1, o2]
        for i, (c, w) in enumerate(((3.6, 0.75), (4.5, 1.0))):
            fw = np.linspace(c - 0.6 * w, c + 0.6 * w, 50)
            o = Observation(f"irac{i + 1}", "photometry", [[c - 0.5 * w, c + 0.5 * w]], np.ones(1), np.ones(1))
            o.filter_response = [list(fw), list(np.where(np.abs(fw - c) <= 0.5 * w, 1.0, 0.02))]
            o.filter_detector_type = "photon"
            obs.append(o)
        pr = syn.eclipse_priors(spec, star_kind, axes)
        rng = np.random.default_rng(spec.seed + (0 if star_kind == "blackbody" else 1 if star_kind == "file" else 2))
        rows = syn.cube_to_physical(pr, rng.uniform(0.05, 0.95, (3, len(pr))))
        rows = np.concatenate([rows, np.zeros((3, 1))], axis=1)   # shift
        rows[1, -1] = 15.0
        if star_kind == "grid":
            rows[1, 2:5] = [4600.0, 4.5, 0.0]       # exactly on grid nodes
            rows[2, 2:5] = [6500.0, 3.0, 0.25]      # T_eff and log g outside: clamped to the edges
        bad = rows[0].copy()
        bad[[p.description for p in pr].index("T0")] = 40.0  # the profile below 50 K: neglected
        params = np.vstack([rows, bad])
        make(name, spec, "secondary_eclipse", same, obs, params, [0, 1, 2], attach_kind="transmission",
             model_cfg=mc, star=star)


if __name__ == "__main__":
    main()
