"""Readers of the result files the solver writes in the reference's formats.

``read_geo`` / ``read_data`` read the binary pair tec/geo and tec/data as the reference's
post-processor does (postCycas.py:readBuf): one record per partition, each with its own
header, until the record of the last partition.  ``read_tecplot`` reads an ASCII FEBRICK
BLOCK file (tec/res0000.dat) and ``read_backup`` a restart file (res.sav).
"""
from __future__ import annotations

import re

import numpy as np


def read_geo(path: str):
    """Partitions of tec/geo: list of (vertices [nvrt, 3], one-based connectivity [ncel, 8])."""
    buf = open(path, "rb").read()
    out, pos = [], 0
    while pos < len(buf):
        rank, nproc, nc, nv = np.frombuffer(buf, dtype="<i4", count=4, offset=pos)
        pos += 16
        vert = np.frombuffer(buf, dtype="<f8", count=3 * nv, offset=pos).reshape(nv, 3)
        pos += 24 * nv
        conn = np.frombuffer(buf, dtype="<i4", count=8 * nc, offset=pos).reshape(nc, 8)
        pos += 32 * nc
        out.append((vert.copy(), conn.copy()))
        if rank == nproc - 1:
            break
    return out


def read_data(path: str, cells_per_partition):
    """Partitions of tec/data: list of arrays [nvar, ncel] (P U V W R T [TE ED]);
    ``cells_per_partition`` gives each record's cell count (from tec/geo)."""
    buf = open(path, "rb").read()
    out, pos = [], 0
    for nc in cells_per_partition:
        rank, nvar = np.frombuffer(buf, dtype="<i4", count=2, offset=pos)
        pos += 8
        out.append(np.frombuffer(buf, dtype="<f8", count=nvar * nc, offset=pos).reshape(nvar, nc).copy())
        pos += 8 * nvar * nc
    return out


def read_tecplot(path: str):
    """ASCII FEBRICK BLOCK zone: dict with ``vert`` [nvrt, 3], ``conn`` one-based [ncel, 8] and
    every cell-centred variable by its name in the header."""
    with open(path) as f:
        head = f.readline()
        zone = f.readline()
        names = re.findall(r'"([^"]*)"', head)
        m = re.search(r"\bN=(\d+),\s*E=(\d+)", zone)
        nv, nc = int(m.group(1)), int(m.group(2))
        tokens = f.read().split()
    vals = tokens[: 3 * nv + (len(names) - 3) * nc]
    a = np.array(vals, dtype=np.float64)
    out = {"vert": np.stack([a[0:nv], a[nv:2 * nv], a[2 * nv:3 * nv]], axis=1)}
    pos = 3 * nv
    for nm in names[3:]:
        out[nm] = a[pos:pos + nc]
        pos += nc
    out["conn"] = np.array(tokens[len(vals):len(vals) + 8 * nc], dtype=np.int64).reshape(nc, 8)
    return out


def read_backup(path: str, ncel: int, turb: int):
    """res.sav: dict of R U V W P T VisLam [VisTur TE ED], each [ncel]."""
    a = np.array(open(path).read().split(), dtype=np.float64)
    per = 11 if turb == 1 else 8
    a = a[: per * ncel].reshape(ncel, per)
    names = ["R", "U", "V", "W", "P", "T", "R", "VisLam"] + (["VisTur", "TE", "ED"] if turb == 1 else [])
    out = {}
    for j, nm in enumerate(names):
        out[nm] = a[:, j].copy()
    return out
