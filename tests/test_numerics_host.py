"""Accuracy of the engine's hand-written exponentials, measured on the CPU.

dfloat.cuh / physics.cuh compile on the host with BGB_HOST_EMULATION (the same
operation sequence in IEEE round-to-nearest host arithmetic, FMA where the
device code uses FMA); tests/numerics_harness.cpp measures each routine
against long-double references over the argument ranges the kernels use:

* exp_tang2048: Tang's table-driven FP64 exp (2048-entry table; the form with
  the table index chosen in FP64);
* exp_tang2048_f: the same with the table index chosen in FP32 from d2f_trunc,
  the exp(-delta) of the short-characteristics recurrence (ulp bound over
  delta <= 40, where a >= 4e-18; relative bound over delta <= 700);
* d2f_trunc: float estimate of a double from its bits (2^-23);
* df_exp2 / 10^x: double-float exponentials of the opacity assembly;
* planck_df: the double-float Planck function;
* df_recip: double-float reciprocal by one Newton step (1/tau, 1/(1 - u) of Planck);
* df_from_double_bits: FP64 value split into a double-float with integer operations
  (the adjoint's stored intensities), identical to df_from_double outside its range;
* df_exp_neg: the double-float exp(-delta) of the adjoint;
* exp_neg_df: the FP64 exp(-delta) of the recurrence from a double-float delta (argument
  reduction in double-float, one FP64 conversion add and FMA), relative error per unit of
  delta (the reduction's low part is rounded once: ~2^-47 delta) and ulp for thin layers;
* f2d_bits / i2d_bits: float and int to double built with integer operations
  (bit-identical to the conversions, checked on every exponent, zeros and subnormals).

The bounds are the accuracy figures the kernels rely on (about 1 ulp for the
FP64 routines; the double-float ones are limited by their ~48-bit inputs).
"""

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))

BOUNDS = {
    "exp_tang2048": 3.4e-16,
    "exp_tang2048_ulp": 1.5,
    "exp_tang2048_f": 3.4e-16,
    "exp_tang2048_f_ulp": 1.5,
    "d2f_trunc": 1.2e-7,        # 2^-23
    "df_recip": 3e-14,          # one Newton step from a float reciprocal (~2^-45)
    "df_from_double_bits": 3.6e-15,   # 2^-48
    "df_from_double_bits_failures": 0,  # outside its range identical to df_from_double
    "df_exp2_edge_failures": 0,  # |y| beyond the clamp: 0 / infinite in the callers; NaN propagates
    "df_exp2": 5e-14,
    "df_pow10": 2e-12,          # |x| <= 40: 10^x from a 48-bit x log2(10)
    "df_exp_neg": 1e-12,        # d <= 60
    "planck_df": 1e-11,         # x = h nu c / k T up to 690: ~x 2^-48 from the 48-bit exponent
    "conversion_mismatches": 0,  # float / int -> double on the integer pipe: bit-identical
    "exp_neg_df_per_d": 1.5e-14,  # relative error / max(delta, 1), delta <= 700: the rounding of the
                                  # reduced argument's low part (~2^-47 delta); the double-float delta
                                  # (a product of the layer depth) carries about as much
    "exp_neg_df_thin_ulp": 1.5,  # delta < 1e-3
}


@pytest.fixture(scope="module")
def measured(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("numerics") / "numerics_harness")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe,
                    os.path.join(HERE, "numerics_harness.cpp")], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    return {k: float(v) for k, v in (line.split() for line in out.strip().splitlines())}


@pytest.mark.parametrize("name", sorted(BOUNDS))
def test_exponential_accuracy(measured, name):
    assert measured[name] <= BOUNDS[name], (name, measured[name])
