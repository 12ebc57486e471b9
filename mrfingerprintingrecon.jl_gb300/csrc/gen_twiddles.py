"""Generates twiddles.cuh: __constant__ tables exp(2 pi i m / R) for the
register DFT base lengths (values computed in float64, rounded to float32), and
the same values as IEEE half bit patterns (constexpr, round to nearest even)
for the fp16 register DFTs."""
import math
import struct
from pathlib import Path

import numpy as np

BASES = (32, 24, 20, 30)


def half_bits(v):
    return int(np.array([v], dtype=np.float16).view(np.uint16)[0])


def main():
    lines = ["// Generated by gen_twiddles.py: c_tw<R>[m] = (cos(2 pi m/R), sin(2 pi m/R)), m < R.",
             "#pragma once", "#include <cuda_runtime.h>", "", "namespace mrsr {", ""]
    for R in BASES:
        vals = []
        for m in range(R):
            a = 2.0 * math.pi * m / R
            c, s = math.cos(a), math.sin(a)
            c = 0.0 if abs(c) < 1e-12 else c  # exact zeros at multiples of pi/2
            s = 0.0 if abs(s) < 1e-12 else s
            c32, s32 = (struct.unpack("f", struct.pack("f", v))[0] for v in (c, s))  # round to float32
            vals.append(f"{{{float.hex(c32)}f, {float.hex(s32)}f}}")
        lines.append(f"static __constant__ float2 c_tw{R}[{R}] = {{")
        for i in range(0, R, 4):
            lines.append("    " + ", ".join(vals[i:i + 4]) + ",")
        lines.append("};")
        lines.append("")
    for R in BASES:
        vals = []
        for m in range(R):
            a = 2.0 * math.pi * m / R
            c, s = math.cos(a), math.sin(a)
            c = 0.0 if abs(c) < 1e-12 else c
            s = 0.0 if abs(s) < 1e-12 else s
            hc, hs = half_bits(c), half_bits(s)
            vals.append(f"{{0x{hc | (hc << 16):08x}u, 0x{hs | (hs << 16):08x}u}}")
        lines.append(f"// c_tw{R} as broadcast half2 bit patterns: {{(cos, cos), (sin, sin)}}")
        lines.append(f"static __constant__ unsigned int c_tw{R}_h2[{R}][2] = {{")
        for i in range(0, R, 4):
            lines.append("    " + ", ".join(vals[i:i + 4]) + ",")
        lines.append("};")
        lines.append("")
    lines.append("}  // namespace mrsr")
    Path(__file__).with_name("twiddles.cuh").write_text("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
