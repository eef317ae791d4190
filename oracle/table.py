"""Completion-table semantics by enumeration (test infrastructure only).

entries(...)   {(fingerprint, label): least subset size} over every column subset of size <= k,
               keyed as cdist/gmitm.c:46-48 (compact: 47-bit fingerprint of zl, 16-bit label) or
               :115 (wide: 63-bit fingerprint, full label)
lookup(...)    least cost <= R with the probe's fingerprint and another label (cdist/gmitm.c:138-163)
"""
from __future__ import annotations

import itertools

FP_COMPACT = 0x7FFFFFFFFFFF0000


def entries(zh, zl, lg, k, wide=False):
    out = {}
    n = len(zh)
    for s in range(k + 1):
        for cols in itertools.combinations(range(n), s):
            l = g = 0
            for j in cols:
                l ^= int(zl[j])
                g ^= int(lg[j])
            key = (l | (1 << 63), g) if wide else (l & FP_COMPACT, g & 0xFFFF)
            if key not in out:
                out[key] = s
    return out


def lookup(table, zl, lg, R, wide=False):
    fp = (int(zl) | (1 << 63)) if wide else int(zl) & FP_COMPACT
    lab = int(lg) if wide else int(lg) & 0xFFFF
    best = -1
    for (f, g), c in table.items():
        if f == fp and g != lab and c <= R and (best < 0 or c < best):
            best = c
    return best
