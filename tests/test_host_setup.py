"""Host-side set-up of the engine (no GPU): grid, band edges, convolution windows
and the composite observation operator against the reference's golden outputs;
the C ABI's exported symbols; error reporting."""

import ctypes
import os
import re

import numpy as np
import pytest

import goldenlib
from bear_gb300 import _lib, build
from bear_gb300.retrieval import Engine

CASES = goldenlib.golden_cases()
HEADER = os.path.join(os.path.dirname(build.HERE), "include", "bear_gb300.h")


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    decl = re.findall(r"^\s*(?:const char\*|int|void)\s+(bear_\w+)\s*\(", open(HEADER).read(), re.M)
    assert len(decl) >= 15
    for name in decl:
        assert hasattr(lib, name), name
    assert set(decl) <= set(_lib.EXPORTS), set(decl) - set(_lib.EXPORTS)


@pytest.fixture(scope="module", params=CASES, ids=lambda p: p.split("/")[-1][:-4])
def prepared(request):
    c = goldenlib.Case(request.param)
    e = Engine(c.config_text(), c.observations(), prepare_only=True)
    yield c, e
    e.close()


def test_grid_and_observation_setup(prepared):
    c, e = prepared
    assert np.array_equal(e.wavenumbers, c.arrays["ref_grid"])
    for k in range(e.nobs):
        assert e.observation_setup(k) == c.setup(k)
    assert e.P == c.params.shape[1]
    assert e.M == c.arrays["ref_obs"].shape[1]


def test_observation_operator_reproduces_binning(prepared):
    """W . F (F: the reference's high-resolution spectrum in native units) equals
    the reference's filtered, convolved and bin-integrated spectrum."""
    c, e = prepared
    emission = c.meta["kind"] == "emission"
    eclipse = c.meta["kind"] == "secondary_eclipse"
    if eclipse and c.meta.get("star"):
        pytest.skip("file and grid stars: the binned stellar flux is not recoverable from the outputs")
    wl = 1e4 / e.wavenumbers
    nu = e.wavenumbers
    obs_arrays = c.observations()
    for j, i in enumerate(c.arrays["spectrum_rows"]):
        if c.arrays["ref_neglect"][i]:
            continue
        F = c.arrays["ref_spectrum"][j].copy()
        if emission:
            F = F * wl * wl / 1e4  # undo the per-micron conversion of the returned spectrum
        if eclipse:
            # blackbody star pi B_nu(T_eff) 1e-3; the returned spectrum is F_p / F_s (R_p/R_s)^2 1e6
            h, cl, kb = 6.62606896e-27, 2.99792458e10, 1.3806504e-16
            rr, teff = c.params[i][1], c.params[i][2]
            Fs = 2.0 * h * cl * cl * nu**3 / np.expm1(h * nu * cl / kb / teff) * np.pi * 1e-3
            F = F * Fs / (rr * rr * 1e6)
        internal = np.empty(e.M)
        for r in range(e.M):
            k0, w = e.operator_row(r)
            internal[r] = w @ F[k0:k0 + w.size]
            if eclipse:
                internal[r] = internal[r] / (w @ Fs[k0:k0 + w.size]) * rr * rr * 1e6
        # shift modifiers are applied after binning
        got = goldenlib.user_order_from_internal(obs_arrays, internal)
        ref = c.arrays["ref_obs"][i].copy()
        P = c.params[i]
        npar = e.P - (1 if "error_inflation 1" in c.config_text() else 0)
        off, mods = 0, []
        for o in obs_arrays:
            if o.modifier == "shift_const":
                mods.append((off, o.n))
            off += o.n
        nmod = len(mods)
        for m, (off, n) in enumerate(mods):
            shift = P[npar - nmod + m]
            if shift != 0:
                got[off:off + n] += shift
        assert goldenlib.rel_err(got, ref) < 1e-12


def test_invalid_config_reports_error():
    lib = _lib.load()
    h = ctypes.c_void_p()
    rc = lib.bear_model_create(b"forward_model eclipse\n", 0, ctypes.byref(h))
    assert rc == 4  # BEAR_ERR_UNSUPPORTED
    assert b"not supported" in lib.bear_last_error()
    rc = lib.bear_model_create(b"nb_grid_points 1\n", 0, ctypes.byref(h))
    assert rc == 1
    with pytest.raises(_lib.EngineError):
        Engine("forward_model emission\nnb_grid_points 10\natmos_boundaries 10 1\n", [], prepare_only=True)


def test_missing_table_file_is_reported(tmp_path):
    c = goldenlib.Case(CASES[0])
    text = c.config_text().replace(c.table_root(), str(tmp_path) + "/")
    with pytest.raises(_lib.EngineError) as ei:
        Engine(text, c.observations(), prepare_only=True)
    assert ei.value.code in (1, 2)


def test_eclipse_configuration_errors(tmp_path):
    """Secondary-eclipse set-up: the stellar model is required and checked (the
    reference's selectStellarModel messages), files must exist, grids must be complete."""
    c = [goldenlib.Case(p) for p in CASES if p.endswith("eclipse_blackbody.npz")][0]
    text = c.config_text()
    obs = c.observations()
    no_star = "\n".join(l for l in text.splitlines() if not l.startswith("stellar_spectrum")) + "\n"
    for bad, code in ((no_star, 1), (text.replace("stellar_spectrum blackbody", "stellar_spectrum blackbody 5000"), 1),
                      (text.replace("stellar_spectrum blackbody", "stellar_spectrum phoenix"), 1),
                      (text.replace("stellar_spectrum blackbody", f"stellar_spectrum file {tmp_path}/none.dat"), 2),
                      (text.replace("stellar_spectrum blackbody", f"stellar_spectrum grid {tmp_path}/"), 2),
                      (text.replace("forward_model secondary_eclipse", "forward_model emission"), 1)):
        with pytest.raises(_lib.EngineError) as ei:
            Engine(bad, obs, prepare_only=True)
        assert ei.value.code == code, (bad.splitlines()[-1], ei.value)
    # an incomplete grid: one spectrum line missing
    from bear_gb300 import synthetic as syn
    axes, wl, sp = syn.star_grid([4000.0, 5000.0], [4.5], [0.0], n=200)
    syn.write_star_grid(str(tmp_path / "g") + "/", axes, wl, sp)
    pf = tmp_path / "g" / "grid_parameters.dat"
    lines = pf.read_text().splitlines()
    pf.write_text("\n".join(lines[:-1]) + "\n")
    with pytest.raises(_lib.EngineError) as ei:
        Engine(text.replace("stellar_spectrum blackbody", f"stellar_spectrum grid {tmp_path}/g/"), obs,
               prepare_only=True)
    assert "inconsistent" in str(ei.value)
    # the short name and the parameter count of a file star: [log g, R_p/R_s] + chemistry ...
    wl2, fl2 = syn.star_spectrum(5000.0, n=300)
    syn.write_star_file(str(tmp_path / "s.dat"), wl2, fl2)
    e = Engine(text.replace("forward_model secondary_eclipse", "forward_model se")
               .replace("stellar_spectrum blackbody", f"stellar_spectrum file {tmp_path}/s.dat"), obs,
               prepare_only=True)
    assert e.P == c.params.shape[1] - 1
    e.close()
