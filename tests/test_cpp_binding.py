"""The reference-side C++ binding, compiled.

bear_gb300/binding/gb300_model.h is the ForwardModel subclass a BeAR maintainer adds
(src/forward_model/forward_model.h:61-144, src/retrieval/select_forward_model.cpp:38).
This test compiles tests/binding_check.cpp -- which includes that header and the
reference's own headers -- with the reference's C++11 flags, links it with the
reference's objects (built by oracle/ref/Makefile) and libbeargb300.so, and runs it on
golden cases: the engine model built from the reference's configuration objects must
report the reference model's parameter count, spectral grid and observation sizes. A
compile or link failure fails the test. It needs the reference's sources, which the
build records in oracle/_ref/REFERENCE_DIR (or BEAR_REFERENCE_DIR names); without them
it is skipped.
"""

import glob
import os
import subprocess

import pytest

import goldenlib
import refcase

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_BUILD = os.path.join(REPO, "oracle", "_ref")
CASES = ["emission_edges", "transmission_edges", "eclipse_blackbody", "emission_batched"]


def _reference_dir():
    d = os.environ.get("BEAR_REFERENCE_DIR", "")
    if not d:
        try:
            with open(os.path.join(REF_BUILD, "REFERENCE_DIR")) as f:
                d = f.read().strip()
        except OSError:
            return None
    return d if os.path.isdir(os.path.join(d, "src")) else None


@pytest.fixture(scope="module")
def binary(tmp_path_factory):
    ref = _reference_dir()
    objs = [o for o in glob.glob(os.path.join(REF_BUILD, "obj", "**", "*.o"), recursive=True)
            if os.path.basename(o) != "harness.o"]
    if not ref or not objs:
        pytest.skip("the reference's sources and objects (oracle/ref/Makefile) are not on this machine")
    from bear_gb300 import build

    lib = build.build()
    out = str(tmp_path_factory.mktemp("binding") / "binding_check")
    cuda_lib = os.path.join(os.path.dirname(os.path.dirname(build._nvcc())), "lib64")
    cmd = ["g++", "-std=c++11", "-O1", "-w", "-fopenmp",
           "-I", os.path.join(REPO, "oracle", "ref", "stubs", "anchor", "anchor"), "-I", os.path.join(ref, "src"),
           "-I", os.path.join(REPO, "include"), "-I", os.path.join(REPO, "bear_gb300", "binding"),
           "-I", os.path.join(REPO, "oracle", "ref"),
           os.path.join(REPO, "tests", "binding_check.cpp")] + objs + [
           lib, f"-Wl,-rpath,{os.path.dirname(lib)}", f"-L{cuda_lib}", f"-Wl,-rpath,{cuda_lib}", "-lcudart",
           "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, f"binding does not compile or link:\n{r.stderr[-4000:]}"
    return out


@pytest.mark.parametrize("name", CASES)
def test_binding_matches_the_reference_model(binary, name, tmp_path):
    c = goldenlib.Case(os.path.join(goldenlib.GOLDEN_DIR, f"{name}.npz"))
    d = str(tmp_path) + "/"
    refcase.write_case(d, c.config_text(), c.observations(), c.params)
    r = subprocess.run([binary, d], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "binding ok" in r.stdout, r.stdout[-3000:] + r.stderr[-3000:]
    params = [ln.split() for ln in r.stdout.splitlines() if ln.startswith("parameters")][0]
    assert int(params[1]) == int(params[2]) == c.params.shape[1] - (1 if "error_inflation 1" in c.config_text() else 0)
