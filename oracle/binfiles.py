"""Reader of the reference's binary snapshots (test infrastructure).

Parses the files CNRGarray / CNRGbasisarray / CNRGmatrix ::SaveBin write
(NRGarrayClass.cpp:780-868, 1947-2003; NRGmatrixClass.cpp:957-1015): counts
are 4-byte ints followed by the elements (int 4 bytes, double 8, complex 16,
bool 1).
"""
from __future__ import annotations

import struct

import numpy as np


def read_bin(path: str, kind: str) -> dict:
    """kind: 'array' (CNRGarray), 'basis' (CNRGbasisarray) or 'matrix' (CNRGmatrix)."""
    b = open(path, "rb").read()
    pos = 0

    def i32():
        nonlocal pos
        v = struct.unpack_from("<i", b, pos)[0]
        pos += 4
        return v

    def vec(dtype, size):
        nonlocal pos
        n = i32()
        v = np.frombuffer(b, dtype, n, pos).copy()
        pos += size * n
        return v

    out = {"Nshell": i32(), "NQNumbers": i32()}
    out["QNumbers"] = vec("<f8", 8)
    out["dEn"] = vec("<f8", 8)
    out["dEigVec"] = vec("<f8", 8)
    out["cEigVec"] = vec("<c16", 16)
    out["BlockBegEnd"] = vec("<i4", 4)
    out["iDegen"] = vec("<i4", 4)
    out["Kept"] = vec("u1", 1)
    out["totalS"] = b[pos]
    pos += 1
    out["Sqnumbers"] = vec("<i4", 4)
    if kind == "basis":
        out["iType"] = vec("<i4", 4)
        out["StCameFrom"] = vec("<i4", 4)
        out["BlockBegEndBC"] = vec("<i4", 4)
        out["BlockBegEndEigVec"] = vec("<i4", 4)
        out["NQNumbers_stcf"] = i32()
        out["StCameFromQNumbers"] = vec("<f8", 8)
    elif kind == "matrix":
        out["MatEl"] = vec("<f8", 8)
        out["MatElCplx"] = vec("<c16", 16)
        out["MatBlockMap"] = vec("<i4", 4)
        out["MatBlockBegEnd"] = vec("<i4", 4)
        out["NeedOld"], out["UpperTriangular"], out["IsComplex"] = b[pos], b[pos + 1], b[pos + 2]
        pos += 3
        out["WignerEckartL"] = struct.unpack_from("<d", b, pos)[0]
        pos += 8
    out["trailing_bytes"] = len(b) - pos
    return out
