"""Generates exp64_table.cuh: constants of the table-driven FP64 exponential and logarithm.

exp: Tang, "Table-driven implementation of the exponential function in IEEE floating-point
arithmetic", ACM TOMS 15(2), 1989 — here with 64 table entries:
x = (64 m + j) ln2/64 + r, |r| <= ln2/128, exp(x) = 2^m * 2^(j/64) * exp(r).
log: Tang, "Table-driven implementation of the logarithm function in IEEE floating-point
arithmetic", ACM TOMS 16(4), 1990 — 64 breakpoints c_j = 1 + (j + 1/2)/64 on [1, 2):
x = 2^e m, log x = e ln2 + log c_j + log1p(m/c_j - 1), |m/c_j - 1| < 1/128.
The constants are computed from their mathematical definitions with mpmath.
"""
import os
import mpmath as mp

mp.mp.dps = 50


def dbl(x):
    return float(x)


def main(path):
    ln2_64 = mp.log(2) / 64
    # Cody-Waite split: L1 keeps 36 significant bits so N*L1 is exact for |N| < 2^17
    L1 = float(ln2_64)
    import struct
    b = struct.unpack("<Q", struct.pack("<d", L1))[0]
    b &= ~((1 << (52 - 35)) - 1)
    L1 = struct.unpack("<d", struct.pack("<Q", b))[0]
    L2 = float(ln2_64 - mp.mpf(L1))
    inv = float(64 / mp.log(2))
    tab = [float(mp.power(2, mp.mpf(j) / 64)) for j in range(64)]
    with open(path, "w") as f:
        f.write("// GENERATED by pelelm_gb300/csrc/gen_exp64.py. Do not edit.\n")
        f.write("#pragma once\n")
        f.write(f"#define PGB_EXP64_INV_LN2_64 {inv!r}\n")
        f.write(f"#define PGB_EXP64_L1 {L1!r}\n")
        f.write(f"#define PGB_EXP64_L2 {L2!r}\n")
        f.write("#define PGB_EXP64_TABLE {" + ", ".join(repr(t) for t in tab) + "}\n")
        cj = [1 + (mp.mpf(j) + mp.mpf(1) / 2) / 64 for j in range(64)]
        f.write("#define PGB_LOG64_INVC {" + ", ".join(repr(float(1 / c)) for c in cj) + "}\n")
        f.write("#define PGB_LOG64_LOGC {" + ", ".join(repr(float(mp.log(c))) for c in cj) + "}\n")
        ln2 = mp.log(2)
        ln2_hi = float(ln2)
        b = struct.unpack("<Q", struct.pack("<d", ln2_hi))[0] & ~((1 << 21) - 1)
        ln2_hi = struct.unpack("<d", struct.pack("<Q", b))[0]
        f.write(f"#define PGB_LOG64_LN2_HI {ln2_hi!r}\n")
        f.write(f"#define PGB_LOG64_LN2_LO {float(ln2 - mp.mpf(ln2_hi))!r}\n")


if __name__ == "__main__":
    main(os.path.join(os.path.dirname(os.path.abspath(__file__)), "gen", "exp64_table.cuh"))
