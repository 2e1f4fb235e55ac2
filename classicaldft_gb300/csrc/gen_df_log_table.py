"""Writes cdft_df_log_table.h: the double-float table of the table-driven logarithm
(cdft_df64.cuh): for F = 1 + j/128, j = -32..64, log F and 1/F as float pairs
(hi = the float nearest the value, lo = the float nearest the rest), from 50-digit
decimal arithmetic. Run: python gen_df_log_table.py > cdft_df_log_table.h
"""
from decimal import Decimal, getcontext

import numpy as np

getcontext().prec = 50
LO, N = -32, 97


def split(x):
    hi = np.float32(float(x))
    lo = np.float32(float(x - Decimal(float(hi))))
    return hi, lo


def lit(f):
    return "%.9ef" % float(f)


print("// Generated by gen_df_log_table.py: {log F hi, log F lo, 1/F hi, 1/F lo} for F = 1 + j/128,")
print("// j = %d..%d (the table of df_log1p in cdft_df64.cuh)." % (LO, LO + N - 1))
print("#pragma once")
print("#define CDFT_DF_LOG_TABLE \\")
rows = []
for i in range(N):
    F = 1 + Decimal(i + LO) / 128
    a, b = split(F.ln())
    c, d = split(1 / F)
    rows.append("  {%s, %s, %s, %s}" % (lit(a), lit(b), lit(c), lit(d)))
print(", \\\n".join(rows))
