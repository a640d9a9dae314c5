"""Restatement of the reference's state record formats (test infrastructure only).

ToolsCore_v_2.0/io_module.f90: RecordLambdas (:191-220), RecordGammas (:222-264),
RecordLabel (:267-287) and the matching readers (:289-472).  One record is one
text line.  Kind 'S' writes each real with the Fortran edit descriptor E30.15
(0.ddd...ddE+xx, 15 significant digits, right-justified in 30 columns; an
exponent beyond +-99 is written as +-xxx without the E); kind 'B' with B80 (the
64-bit pattern in binary without leading zeros, right-justified in 80 columns).
Labels use I16.  Written independently of the library's C++ (io.cu) so that the
tests can compare the two byte for byte.
"""
from __future__ import annotations

import struct

import numpy as np


def e30_15(x: float) -> str:
    if x != x:
        body = "NaN"
    elif x in (float("inf"), float("-inf")):
        body = "-Infinity" if x < 0 else "Infinity"
    elif x == 0.0:
        body = ("-" if np.signbit(x) else "") + "0.000000000000000E+00"
    else:
        m = "%.14E" % abs(x)                      # d.dddddddddddddd E+xx
        mant, ex = m.split("E")
        e10 = int(ex) + 1                         # 0.d1d2... x 10^e10
        digits = mant.replace(".", "")
        exp = ("E%+03d" % e10) if -99 <= e10 <= 99 else ("%+04d" % e10)
        body = ("-" if x < 0 else "") + "0." + digits + exp
    return body.rjust(30)


def b80(x: float) -> str:
    u = struct.unpack("<Q", struct.pack("<d", float(x)))[0]
    return format(u, "b").rjust(80)


def _real(x, kind):
    return e30_15(x) if kind == "S" else b80(x)


def format_lambdas(lambdas, kind="S") -> str:
    return "".join("".join(_real(v, kind) for v in l) + "\n" for l in lambdas)


def format_gammas(gammas, kind="S") -> str:
    out = []
    for part in (np.real, np.imag):
        for g in gammas:
            chi, d, _ = g.shape
            p = part(g)
            for i in range(chi):
                for j in range(chi):
                    out.append("".join(_real(p[i, k, j], kind) for k in range(d)) + "\n")
    return "".join(out)


def format_labels(labels) -> str:
    return "".join("".join("%16d" % v for v in l) + "\n" for l in labels)


def _field(s: str, kind: str) -> float:
    s = s.strip()
    if kind == "B":
        return struct.unpack("<d", struct.pack("<Q", int(s, 2)))[0]
    s = s.replace("D", "E")
    if "E" not in s:
        p = max(s.rfind("+"), s.rfind("-"))
        s = s[:p] + "E" + s[p:]
    return float(s)


def parse_lambdas(text: str, L: int, chi: int, kind="S"):
    w = 30 if kind == "S" else 80
    lines = text.splitlines()
    return [np.array([_field(lines[l][w * j:w * (j + 1)], kind) for j in range(chi)]) for l in range(L + 1)]


def parse_gammas(text: str, L: int, chi: int, d: int, kind="S"):
    w = 30 if kind == "S" else 80
    lines = iter(text.splitlines())
    gam = [np.zeros((chi, d, chi), complex, order="F") for _ in range(L)]
    for part in (1.0, 1j):
        for g in gam:
            for i in range(chi):
                for j in range(chi):
                    line = next(lines)
                    for k in range(d):
                        g[i, k, j] += part * _field(line[w * k:w * (k + 1)], kind)
    return gam
