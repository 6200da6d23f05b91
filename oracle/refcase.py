"""Runs the reference's own CPU path (oracle/_ref/bear_ref_harness, built from
the reference sources by oracle/ref/Makefile) on a case and reads back its
outputs. Test infrastructure: used to generate golden vectors and to pin the C
oracle; never part of the product path.
"""

from __future__ import annotations

import os
import subprocess
from typing import List, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
HARNESS = os.path.join(HERE, "_ref", "bear_ref_harness")


def available() -> bool:
    return os.path.exists(HARNESS)


def write_case(case_dir: str, config_text: str, observations, params: np.ndarray) -> None:
    """observations: list of bear_gb300.config.ObservationArrays."""
    os.makedirs(case_dir, exist_ok=True)
    with open(os.path.join(case_dir, "config.txt"), "w") as f:
        f.write(config_text)
    with open(os.path.join(case_dir, "observations.txt"), "w") as f:
        for o in observations:
            nf = 0 if o.filter_wavelength is None else len(o.filter_wavelength)
            f.write("observation {} {} {} {} {} {} {} {}\n".format(
                o.name, o.type, o.n, int(o.fwhm is not None), int(o.weight is not None), nf,
                o.detector or "-", o.modifier or "-"))
            for i in range(o.n):
                row = []
                if o.centers_or_edges.ndim == 1:
                    row.append(repr(float(o.centers_or_edges[i])))
                else:
                    row += [repr(float(o.centers_or_edges[i, 0])), repr(float(o.centers_or_edges[i, 1]))]
                row += [repr(float(o.data[i])), repr(float(o.error[i]))]
                if o.fwhm is not None:
                    row.append(repr(float(o.fwhm[i])))
                if o.weight is not None:
                    row.append(repr(float(o.weight[i])))
                f.write(" ".join(row) + "\n")
            for i in range(nf):
                f.write(f"{float(o.filter_wavelength[i])!r} {float(o.filter_response[i])!r}\n")
    params = np.atleast_2d(np.asarray(params, dtype=np.float64))
    with open(os.path.join(case_dir, "params.txt"), "w") as f:
        f.write(f"{params.shape[1]} {params.shape[0]}\n")
        for row in params:
            f.write(" ".join(repr(float(x)) for x in row) + "\n")


def run_case(case_dir: str, repeat: int = 0, threads: int = 0) -> dict:
    env = dict(os.environ)
    if threads:
        env["OMP_NUM_THREADS"] = str(threads)
    cmd = [HARNESS, case_dir]
    if repeat:
        cmd += ["--repeat", str(repeat)]
    res = subprocess.run(cmd, capture_output=True, text=True, env=env)
    if res.returncode != 0:
        raise RuntimeError(f"reference harness failed ({res.returncode}):\n{res.stdout[-3000:]}\n{res.stderr[-3000:]}")
    out = {
        "grid": np.fromfile(os.path.join(case_dir, "ref_grid.bin"), dtype=np.float64),
        "loglike": np.fromfile(os.path.join(case_dir, "ref_loglike.bin"), dtype=np.float64),
        "neglect": np.fromfile(os.path.join(case_dir, "ref_neglect.bin"), dtype=np.float64),
    }
    S = out["loglike"].size
    out["spectrum"] = np.fromfile(os.path.join(case_dir, "ref_spectrum.bin"), dtype=np.float64).reshape(S, -1)
    out["obs"] = np.fromfile(os.path.join(case_dir, "ref_obs.bin"), dtype=np.float64).reshape(S, -1)
    setup: List[dict] = []
    with open(os.path.join(case_dir, "ref_setup.txt")) as f:
        for line in f:
            t = line.split()
            if t[0] == "observation":
                setup.append({"n": int(t[1]), "range": (int(t[2]), int(t[3])), "filter_norm": float(t[4]),
                              "edges": [], "conv": []})
            elif t[0] == "edge":
                setup[-1]["edges"].append((int(t[1]), int(t[2])))
            elif t[0] == "conv":
                setup[-1]["conv"].append((int(t[1]), int(t[2])))
    out["setup"] = setup
    for line in res.stdout.splitlines():
        if line.startswith("ref_seconds_per_eval"):
            out["seconds_per_eval"] = float(line.split()[1])
    out["stdout"] = res.stdout
    return out


def run_priors(case_dir: str, config_text: str, observations, priors, cube: np.ndarray) -> dict:
    """Retrieval::convertCubeParameters of the reference (harness --priors) for every row
    of ``cube`` with the given prior list (bear_gb300.config.Prior: type, description,
    parameter, unit) on the model of ``config_text`` / ``observations``."""
    cube = np.atleast_2d(np.asarray(cube, dtype=np.float64))
    write_case(case_dir, config_text, observations, cube)
    with open(os.path.join(case_dir, "priors.txt"), "w") as f:
        for p in priors:
            vals = " ".join(repr(float(x)) for x in p.parameter)
            f.write(f"{p.type} {p.description.replace(' ', '_')} {p.unit or '-'} {len(p.parameter)} {vals}\n")
    with open(os.path.join(case_dir, "cube.txt"), "w") as f:
        f.write(f"{cube.shape[1]} {cube.shape[0]}\n")
        for row in cube:
            f.write(" ".join(repr(float(x)) for x in row) + "\n")
    res = subprocess.run([HARNESS, case_dir, "--priors"], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"reference harness failed ({res.returncode}):\n{res.stdout[-3000:]}\n{res.stderr[-3000:]}")
    S, P = cube.shape
    return {"parameter": np.fromfile(os.path.join(case_dir, "ref_prior_parameter.bin"), dtype=np.float64).reshape(S, P),
            "physical": np.fromfile(os.path.join(case_dir, "ref_prior_physical.bin"), dtype=np.float64).reshape(S, P)}
