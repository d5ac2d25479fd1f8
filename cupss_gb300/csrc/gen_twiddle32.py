"""Writes twiddle32.h: exp(-2*pi*i*j/64), j in [0,64), and exp(-2*pi*i*j/192), j in
[0,192), as exact float hex literals.

The register-level DFTs (radix <= 64, or 3 * 2^b <= 192) and the compile-time twiddle
factors of the row passes take their twiddles from these tables at compile time.  Values
are computed in double and rounded once to float (entry 2j of a table equals the entry j
of the table of half the order exactly: the double arguments are the same).
"""
import math
import os
import struct


def f32hex(v):
    if abs(v) < 1e-12:          # exact zeros at multiples of pi/2
        v = 0.0
    f = struct.unpack("f", struct.pack("f", v))[0]
    return float(f).hex() + "f" if f != 0.0 else "0.0f"


lines = ["// Generated by gen_twiddle32.py -- do not edit.",
         "#pragma once",
         "namespace cupssgb {",
         "// kTw64Re[j] + i*kTw64Im[j] = exp(-2*pi*i*j/64)",
         "constexpr float kTw64Re[64] = {"]
lines.append(", ".join(f32hex(math.cos(2 * math.pi * j / 64)) for j in range(64)) + "};")
lines.append("constexpr float kTw64Im[64] = {")
lines.append(", ".join(f32hex(-math.sin(2 * math.pi * j / 64)) for j in range(64)) + "};")
lines.append("// kTw192Re[j] + i*kTw192Im[j] = exp(-2*pi*i*j/192)")
lines.append("constexpr float kTw192Re[192] = {")
lines.append(", ".join(f32hex(math.cos(2 * math.pi * j / 192)) for j in range(192)) + "};")
lines.append("constexpr float kTw192Im[192] = {")
lines.append(", ".join(f32hex(-math.sin(2 * math.pi * j / 192)) for j in range(192)) + "};")
lines.append("}  // namespace cupssgb")
here = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(here, "twiddle32.h"), "w") as fh:
    fh.write("\n".join(lines) + "\n")
