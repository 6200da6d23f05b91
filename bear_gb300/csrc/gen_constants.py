"""Writes dfconst.h: the constants of the engine's exponential routines,
computed to 60 digits with mpmath and split into (hi, lo) pairs.

  2^(j/64), j = -32..32  as float pairs   (double-float exp2, Tang's table method)
  2^(j/2048), j = 0..2047 as doubles      (FP64 exp with a degree-3 polynomial)
  ln 2, log2 10, log2 e  as float pairs; ln2/2048 as a double pair (Cody-Waite)
  ln2/2048               as a float pair (argument reduction in double-float)

Run: python bear_gb300/csrc/gen_constants.py > bear_gb300/csrc/dfconst.h
"""

import struct

import mpmath

mpmath.mp.dps = 60


def f32(x):
    return struct.unpack("f", struct.pack("f", float(x)))[0]


def split_f(x):
    hi = f32(x)
    lo = f32(x - mpmath.mpf(hi))
    return hi, lo


def split_d(x):
    hi = float(x)
    lo = float(x - mpmath.mpf(hi))
    return hi, lo


def ff(v):
    return float(v).hex() + "f" if v != 0 else "0.0f"


print("// Generated by gen_constants.py (mpmath, 60 digits). Do not edit.")
print("#pragma once")
print("#ifdef BGB_HOST_EMULATION\n#define BGB_CONST_MEM static const\n#define BGB_GLOBAL_MEM static const\n#else\n#define BGB_CONST_MEM static __device__ __constant__\n#define BGB_GLOBAL_MEM static __device__ const\n#endif")
print("namespace bgb {")
print("// 2^(j/64) for j = -32..32 as (hi, lo) floats")
print("BGB_CONST_MEM float kExp2TabHi[65] = {" + ", ".join(ff(split_f(mpmath.power(2, mpmath.mpf(j) / 64))[0]) for j in range(-32, 33)) + "};")
print("BGB_CONST_MEM float kExp2TabLo[65] = {" + ", ".join(ff(split_f(mpmath.power(2, mpmath.mpf(j) / 64))[1]) for j in range(-32, 33)) + "};")
print("// 2^(j/2048) for j = 0..2047 as doubles (global memory: blocks stage it in shared memory)")
print("BGB_GLOBAL_MEM double kExp2TabD2048[2048] = {" + ", ".join(float(mpmath.power(2, mpmath.mpf(j) / 2048)).hex() for j in range(2048)) + "};")
for name, val in (("Ln2", mpmath.log(2)), ("Log2_10", mpmath.log(10, 2)), ("Log2e", 1 / mpmath.log(2))):
    hi, lo = split_f(val)
    print(f"constexpr float k{name}Hi = {ff(hi)}, k{name}Lo = {ff(lo)};")
hi, lo = split_d(mpmath.log(2) / 2048)
print(f"constexpr double kLn2Over2048Hi = {hi.hex()}, kLn2Over2048Lo = {lo.hex()};")
print(f"constexpr double k2048OverLn2 = {float(2048 / mpmath.log(2)).hex()};")
hi, lo = split_f(mpmath.log(2) / 2048)
print(f"constexpr float kLn2Over2048FHi = {ff(hi)}, kLn2Over2048FLo = {ff(lo)};")
print("}  // namespace bgb")
