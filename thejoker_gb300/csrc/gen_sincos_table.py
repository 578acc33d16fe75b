"""Writes joker_sincos_table.cuh: sin(k/128) and cos(k/128) for k = 0..403,
each rounded to the nearest double from a 60-digit mpmath evaluation.

The FP64 Kepler solver reads the table to evaluate sin and cos of an FP32
angle in [0, 403/128] to FP64 accuracy.  Run from any directory:

    python thejoker_gb300/csrc/gen_sincos_table.py
"""
import os

import mpmath

N = 404          # k/128 for k = 0..403 covers [0, 3.148] > pi + the starter's error


def main():
    mpmath.mp.dps = 60
    rows = []
    for k in range(N):
        a = mpmath.mpf(k) / 128
        s, c = float(mpmath.sin(a)), float(mpmath.cos(a))
        rows.append(f"    {{{s.hex()}, {c.hex()}}},")
    body = "\n".join(rows)
    text = f"""// Generated by gen_sincos_table.py: sin and cos of k/128 rad, k = 0..{N - 1},
// each the double nearest to the exact value.  Do not edit.
#pragma once
#include <cuda_runtime.h>

namespace joker {{

constexpr int SINCOS_TAB_N = {N};

static __device__ const double2 kSinCos128[SINCOS_TAB_N] = {{
{body}
}};

}}  // namespace joker
"""
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "joker_sincos_table.cuh")
    with open(out, "w") as f:
        f.write(text)
    print(f"wrote {out}")


if __name__ == "__main__":
    main()
