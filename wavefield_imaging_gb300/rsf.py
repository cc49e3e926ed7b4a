"""RSF (Madagascar) file I/O for the drop-in programs' inputs and outputs.

An RSF dataset is a text header of ``key=value`` pairs (``n1 o1 d1 ...``,
``data_format``, ``esize``) plus the samples, which live in the binary file
named by ``in=``.  Axis 1 is the fastest-varying.  Native little-endian
float32 (``data_format=native_float``, ``esize=4``) is what the modelling
programs read and write (``sf_floatread``/``sf_floatwrite`` in
CODE/MAWEFDcart2Dgpu.cu:174, :509); complex64 (``native_complex``,
``esize=8``) is the data type of the point-cloud tools
(CODE/Mbycloudwin3d.c:95, ``sf_complexread``).
"""
from __future__ import annotations

import os
import shlex

import numpy as np


def _parse(text: str) -> dict:
    hdr = {}
    for tok in shlex.split(text, comments=False, posix=True):
        if "=" in tok:
            k, v = tok.split("=", 1)
            hdr[k] = v
    return hdr


def read_header(path: str) -> dict:
    with open(path, "rb") as f:
        raw = f.read()
    # headers that carry their samples inline stop at the 0x0c 0x0c 0x04 mark
    cut = raw.find(b"\x0c\x0c\x04")
    text = (raw if cut < 0 else raw[:cut]).decode("latin-1")
    hdr = _parse(text)
    if cut >= 0:
        hdr["_inline_offset"] = str(cut + 3)
    return hdr


def axes(hdr: dict) -> list[tuple[int, float, float]]:
    """List of (n, o, d) for axes 1..k, dropping trailing unit axes."""
    out = []
    for i in range(1, 10):
        n = int(hdr.get("n%d" % i, 1))
        o = float(hdr.get("o%d" % i, 0.0))
        d = float(hdr.get("d%d" % i, 1.0))
        out.append((n, o, d))
    while len(out) > 1 and out[-1][0] == 1:
        out.pop()
    return out


def read(path: str):
    """Return (array, header).  The array is shaped [nk..n2, n1] (C order,
    axis 1 fastest): float32, or complex64 for native_complex data."""
    hdr = read_header(path)
    fmt = hdr.get("data_format", "native_float").strip('"')
    cplx = fmt == "native_complex" and int(hdr.get("esize", 8)) == 8
    if not cplx and (fmt not in ("native_float", "xdr_float") or int(hdr.get("esize", 4)) != 4):
        raise ValueError("%s: only float32 or complex64 RSF data is supported (got %s)" % (path, fmt))
    dims = [a[0] for a in axes(hdr)]
    count = int(np.prod(dims))
    dt = "<c8" if cplx else ("<f4" if fmt != "xdr_float" else ">f4")
    if "_inline_offset" in hdr:
        data = np.fromfile(path, dtype=dt, count=count, offset=int(hdr["_inline_offset"]))
    else:
        binp = hdr.get("in", "").strip('"')
        if not binp:
            raise ValueError("%s: header has no in=" % path)
        if not os.path.isabs(binp) and not os.path.exists(binp):
            binp = os.path.join(os.path.dirname(os.path.abspath(path)), binp)
        data = np.fromfile(binp, dtype=dt, count=count)
    if data.size != count:
        raise ValueError("%s: expected %d samples, found %d" % (path, count, data.size))
    return data.astype(np.complex64 if cplx else np.float32).reshape(dims[::-1]), hdr


def write(path: str, arr, ax: list[tuple[int, float, float]] | None = None, extra: dict | None = None):
    """Write ``arr`` (C order, last index = axis 1) to ``path`` with binary
    ``path@``: float32 samples, or complex64 (native_complex) when ``arr`` is
    complex.  ``ax`` gives (n, o, d) per axis from axis 1; defaults to the
    array's shape with o=0, d=1."""
    cplx = np.iscomplexobj(arr)
    a = np.ascontiguousarray(arr, dtype=np.complex64 if cplx else np.float32)
    if ax is None:
        ax = [(n, 0.0, 1.0) for n in a.shape[::-1]]
    if int(np.prod([x[0] for x in ax])) != a.size:
        raise ValueError("axes do not match array size")
    binp = os.path.abspath(path) + "@"
    a.astype("<c8" if cplx else "<f4").tofile(binp)
    lines = []
    for i, (n, o, d) in enumerate(ax, start=1):
        lines.append("n%d=%d o%d=%.9g d%d=%.9g" % (i, n, i, o, i, d))
    for k, v in (extra or {}).items():
        lines.append("%s=%s" % (k, v))
    lines.append('data_format="native_complex" esize=8' if cplx else 'data_format="native_float" esize=4')
    lines.append('in="%s"' % binp)
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
