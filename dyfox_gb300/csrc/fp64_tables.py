"""Writes fp64_tables.cuh: the tables of the table-driven double-precision
logarithm and arctangent of volterra.cuh (log_d, atan2_d).

    python dyfox_gb300/csrc/fp64_tables.py

  kLogF[j]  = ln(1 + j/128),  j = 0..128
  kInvF[j]  = 1 / (1 + j/128)
  kAtanC[j] = atan(j/64),     j = 0..64
  kF[j] = 1 + j/128, kAtanX[j] = j/64 (exact)
  kELn2Hi[k] = -k kLn2Hi (exact), kELn2Lo[k] = -k kLn2Lo, k = 0..255
  ln 2 split as kLn2Hi (its leading 42 bits: k kLn2Hi is exact for integer
  |k| < 2^11) + kLn2Lo.

Values from Python's math module (IEEE double, within an ulp), written as
hexadecimal floating literals so the header reproduces them exactly.
"""

import math
import os

HERE = os.path.dirname(os.path.abspath(__file__))


def hexd(v):
    return float(v).hex()


def main():
    ln2 = math.log(2.0)
    m, e = math.frexp(ln2)
    hi = math.ldexp(math.floor(math.ldexp(m, 42)), e - 42)
    lo = ln2 - hi
    rows = ["// Generated by fp64_tables.py: tables of the double-precision",
            "// logarithm and arctangent of volterra.cuh.  Do not edit.",
            "#pragma once", "", "namespace dyfox {", ""]
    rows.append(f"constexpr double kLn2Hi = {hexd(hi)};")
    rows.append(f"constexpr double kLn2Lo = {hexd(lo)};")
    rows.append("")
    rows.append("__device__ const double kLogF[129] = {")
    rows += [f"    {hexd(math.log1p(j / 128.0))}," for j in range(129)]
    rows.append("};")
    rows.append("__device__ const double kInvF[129] = {")
    rows += [f"    {hexd(1.0 / (1.0 + j / 128.0))}," for j in range(129)]
    rows.append("};")
    rows.append("__device__ const double kAtanC[65] = {")
    rows += [f"    {hexd(math.atan(j / 64.0))}," for j in range(65)]
    rows.append("};")
    # exact table points, read instead of converted from the index
    rows.append("__device__ const double kF[129] = {")
    rows += [f"    {hexd(1.0 + j / 128.0)}," for j in range(129)]
    rows.append("};")
    rows.append("__device__ const double kAtanX[65] = {")
    rows += [f"    {hexd(j / 64.0)}," for j in range(65)]
    rows.append("};")
    # e ln 2 for e = 0, -1, ..., -255: e kLn2Hi (exact) and e kLn2Lo
    rows.append("__device__ const double kELn2Hi[256] = {")
    rows += [f"    {hexd(-e * hi)}," for e in range(256)]
    rows.append("};")
    rows.append("__device__ const double kELn2Lo[256] = {")
    rows += [f"    {hexd(-e * lo)}," for e in range(256)]
    rows.append("};")
    rows += ["", "}  // namespace dyfox", ""]
    with open(os.path.join(HERE, "fp64_tables.cuh"), "w") as f:
        f.write("\n".join(rows))


if __name__ == "__main__":
    main()
