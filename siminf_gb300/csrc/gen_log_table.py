"""Generate the constants of the logarithm (``si_log``) and exponential
(``si_exp``) in siminf_stream.h.

The logarithm is evaluated as ln(x) = K*ln(2) + L_j + ln(1 + z), where
x = 2^e * f, f in [1, 2), j = the top 7 fraction bits of f, and
z = f * R_j / 2^10 - 1 is exact in 64-bit integer arithmetic because
R_j has at most 11 bits.  This script prints R_j, L_j = ln(2^10 / R_j)
in Q64, ln(2) to 128 bits and the Q62 Taylor coefficients of
ln(1+z)/z = sum_i (-1)^i z^i / (i+1), using mpmath at 200 bits so the
constants are correctly rounded.

Run:  python siminf_gb300/csrc/gen_log_table.py > siminf_gb300/csrc/siminf_log_table.h
"""
import mpmath as mp

mp.mp.prec = 200


def q(x, bits):
    return int(mp.nint(x * mp.mpf(2) ** bits))


def main():
    R, L, D = [], [], []
    for j in range(128):
        if j == 0:
            r, d = 1024, 0           # f in [1, 1+1/128): z = f - 1 exactly
        elif j == 127:
            r, d = 512, 1            # f in [2-1/128, 2): ln f = ln 2 + ln(f/2)
        else:
            c = 1 + (mp.mpf(j) + mp.mpf("0.5")) / 128
            r, d = int(mp.nint(1024 / c)), 0
        R.append(r)
        D.append(d)
        lj = mp.log(mp.mpf(1024) / r) - d * mp.log(2)
        L.append(q(lj, 64))
    ln2 = q(mp.log(2), 128)
    coef = [q(mp.mpf((-1) ** i) / (i + 1), 62) for i in range(9)]
    # si_exp: ln 2 split into a 32-significant-bit head (k * head is exact for
    # |k| < 2^21) and the double nearest to the rest; 1/ln 2; 1/n! for the
    # Taylor series of exp on |r| <= ln(2)/2.
    ln2f = mp.log(2)
    e = mp.floor(mp.log(ln2f, 2))
    head = mp.floor(ln2f / mp.mpf(2) ** (e - 31)) * mp.mpf(2) ** (e - 31)
    tail = ln2f - head
    import struct

    def dbits(x):
        return struct.unpack("<Q", struct.pack("<d", float(x)))[0]
    exp_consts = {"SI_EXP_LN2_HI": dbits(head), "SI_EXP_LN2_LO": dbits(tail),
                  "SI_EXP_INV_LN2": dbits(1 / ln2f)}
    inv_fact = [dbits(1 / mp.factorial(n)) for n in range(14)]
    # si_neglog_u32: two-level reduction tables for x = 2w+1 < 2^33.
    # Level 1: m in [1, 2) (Q32, M in [2^32, 2^33)), j1 = top 7 fraction bits,
    # R1 = round(2^10 / c1), c1 the bucket centre; L1 = ln(2^10 / R1) in Q64.
    # Level 2: z1 = M*R1/2^42 - 1 in [-2^-7, 2^-7), j2 = bucket of width
    # 2^-14, R2 = round(2^16 / (1 + centre)); L2 = ln(2^16 / R2) in Q64 (signed).
    R1, L1 = [], []
    for j in range(128):
        c = 1 + (mp.mpf(j) + mp.mpf("0.5")) / 128
        r = int(mp.nint(1024 / c))
        R1.append(r)
        L1.append(q(mp.log(mp.mpf(1024) / r), 64))
    R2, L2 = [], []
    for j in range(256):
        lo = -mp.mpf(2) ** -7 + mp.mpf(j) * mp.mpf(2) ** -14
        c = 1 + lo + mp.mpf(2) ** -15
        r = int(mp.nint(mp.mpf(2) ** 16 / c))
        R2.append(r)
        L2.append(q(mp.log(mp.mpf(2) ** 16 / r), 64))
    KLN2 = [q(k * mp.log(2), 64) for k in range(34)]
    out = []
    out.append("/* Generated by gen_log_table.py: constants of si_log (do not edit). */")
    out.append("#ifndef SIMINF_LOG_TABLE_H")
    out.append("#define SIMINF_LOG_TABLE_H")
    out.append("#define SI_LN2_Q128_HI 0x%016xULL" % (ln2 >> 64))
    out.append("#define SI_LN2_Q128_LO 0x%016xULL" % (ln2 & (2 ** 64 - 1)))
    out.append("/* R_j | (delta_j << 16): reciprocal of the bucket centre in Q10. */")
    out.append("#define SI_LOG_R_INIT { \\")
    for i in range(0, 128, 8):
        out.append("    " + ", ".join("0x%05xu" % (R[k] | (D[k] << 16)) for k in range(i, i + 8)) + ", \\")
    out.append("}")
    out.append("/* L_j = ln(2^10 / R_j) - delta_j ln 2 in Q64 (unsigned, 0 <= L_j < 1). */")
    out.append("#define SI_LOG_L_INIT { \\")
    for i in range(0, 128, 4):
        out.append("    " + ", ".join("0x%016xULL" % L[k] for k in range(i, i + 4)) + ", \\")
    out.append("}")
    out.append("/* (-1)^i / (i+1) in Q62, i = 0..8. */")
    for i, c in enumerate(coef):
        if c < 0:
            out.append("#define SI_LOG_C%d (-(int64_t)0x%016xLL)" % (i, -c))
        else:
            out.append("#define SI_LOG_C%d ((int64_t)0x%016xLL)" % (i, c))
    for k, v in exp_consts.items():
        out.append("#define %s 0x%016xULL" % (k, v))
    out.append("/* 1/n!, n = 0..13, as IEEE double bits. */")
    out.append("#define SI_EXP_INV_FACT_INIT { \\")
    for i in range(0, 14, 4):
        out.append("    " + ", ".join("0x%016xULL" % inv_fact[k] for k in range(i, min(i + 4, 14))) + ", \\")
    out.append("}")
    out.append("/* si_neglog_u32 tables. */")
    out.append("#define SI_NL_R1_INIT { \\")
    for i in range(0, 128, 8):
        out.append("    " + ", ".join("%du" % R1[k] for k in range(i, i + 8)) + ", \\")
    out.append("}")
    out.append("#define SI_NL_L1_INIT { \\")
    for i in range(0, 128, 4):
        out.append("    " + ", ".join("0x%016xULL" % L1[k] for k in range(i, i + 4)) + ", \\")
    out.append("}")
    out.append("#define SI_NL_R2_INIT { \\")
    for i in range(0, 256, 8):
        out.append("    " + ", ".join("%du" % R2[k] for k in range(i, i + 8)) + ", \\")
    out.append("}")
    out.append("#define SI_NL_L2_INIT { \\")
    for i in range(0, 256, 4):
        out.append("    " + ", ".join(("-(int64_t)0x%016xLL" % -L2[k]) if L2[k] < 0 else
                                      ("(int64_t)0x%016xLL" % L2[k]) for k in range(i, i + 4)) + ", \\")
    out.append("}")
    out.append("/* k ln 2 in Q64.64, k = 0..33: {integer part, fraction}. */")
    out.append("#define SI_NL_KLN2_INIT { \\")
    for k in range(34):
        out.append("    {0x%xULL, 0x%016xULL}, \\" % (KLN2[k] >> 64, KLN2[k] & (2 ** 64 - 1)))
    out.append("}")
    out.append("#endif")
    print("\n".join(out))


if __name__ == "__main__":
    main()
