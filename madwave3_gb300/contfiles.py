"""Continuation files of the time loop (wvpcont, SRC/main_madwave3.f:496-551,
read back at SRC/main_madwave3.f:218-260, SRC/mod_flux_01y2.f:296-320 and
SRC/mod_coortrans01_02.f:183-197), so a propagation can stop and resume across
the library and the reference:

* ``contNN.paq``: psi_{k-1}, psi_k (two records of FP64),
* ``contNN.S2``: zS2, zCR, zCdR (three records of complex FP64),
* ``contNN.S2prod``: zS2prod (iprod = 2),
* ``cont.data`` (list-directed text): ``iit0 indt+1 iloop`` and
  ``abstot nflux ncan``.

The binary files are Fortran unformatted sequential files as gfortran writes
them: each record is framed by a 4-byte little-endian byte count before and
after it; a record longer than a subrecord's 2147483639 bytes is split into
subrecords whose leading count is negative when the record continues and whose
trailing count is negative when it continued from the previous subrecord.
Arrays keep the Fortran order, which is the C order of the library's
(mw3_download_state / mw3_download_accumulators) arrays.
"""
import os
import struct

import numpy as np

MAX_SUBRECORD = 2147483639


def write_record(f, data, max_sub=MAX_SUBRECORD):
    """One unformatted sequential record (bytes or an array's raw bytes)."""
    b = data.tobytes() if isinstance(data, np.ndarray) else bytes(data)
    n = len(b)
    if n == 0:
        f.write(struct.pack("<i", 0) * 2)
        return
    pieces = [b[i:i + max_sub] for i in range(0, n, max_sub)]
    last = len(pieces) - 1
    for k, p in enumerate(pieces):
        L = len(p)
        f.write(struct.pack("<i", -L if k < last else L))
        f.write(p)
        f.write(struct.pack("<i", -L if k > 0 else L))


def read_record(f):
    """The next record's bytes (subrecords joined); raises EOFError at the end."""
    out = bytearray()
    while True:
        h = f.read(4)
        if len(h) < 4:
            raise EOFError("no record")
        L = struct.unpack("<i", h)[0]
        body = f.read(abs(L))
        t = f.read(4)
        if len(body) != abs(L) or len(t) != 4 or abs(struct.unpack("<i", t)[0]) != abs(L):
            raise ValueError("corrupt record framing")
        out += body
        if L >= 0:
            return bytes(out)


def _complex(a):
    return np.ascontiguousarray(a, np.complex128)


def write_cont(outdir, psi_km1, psi_k, zs2, zcr, zcdr, iit0, indt, iloop, abstot=0.0, idproc=0, zs2prod=None):
    """wvpcont for one process: the four files in outdir.  zs2 [ncan][nj][nv][netot],
    zcr/zcdr [nflux][netot] complex; zs2prod [nom][njp][nvp][netot] complex."""
    with open(os.path.join(outdir, "cont%02d.paq" % idproc), "wb") as f:
        write_record(f, np.ascontiguousarray(psi_km1, np.float64))
        write_record(f, np.ascontiguousarray(psi_k, np.float64))
    with open(os.path.join(outdir, "cont%02d.S2" % idproc), "wb") as f:
        write_record(f, _complex(zs2))
        write_record(f, _complex(zcr))
        write_record(f, _complex(zcdr))
    if zs2prod is not None:
        with open(os.path.join(outdir, "cont%02d.S2prod" % idproc), "wb") as f:
            write_record(f, _complex(zs2prod))
    zcr = np.asarray(zcr)
    ncan = np.asarray(zs2).shape[0]
    with open(os.path.join(outdir, "cont.data"), "w") as f:
        f.write(" %d %d %d\n" % (iit0, indt + 1, iloop))
        f.write(" %r %d %d\n" % (float(abstot), zcr.shape[0], ncan))


def read_cont(outdir, idproc=0, zs2_shape=None, flux_shape=None, prod_shape=None):
    """The continuation files back: dict with iit0, indt, iloop (as cont.data
    holds them), psi_km1, psi_k and, where the shapes are given, zs2, zcr, zcdr,
    zs2prod (complex, reshaped)."""
    out = {}
    with open(os.path.join(outdir, "cont.data")) as f:
        a = f.readline().split()
        out["iit0"], out["indt"], out["iloop"] = int(a[0]), int(a[1]), int(a[2])
        b = f.readline().split()
        out["abstot"], out["nflux"], out["ncan"] = float(b[0]), int(b[1]), int(b[2])
    with open(os.path.join(outdir, "cont%02d.paq" % idproc), "rb") as f:
        out["psi_km1"] = np.frombuffer(read_record(f), np.float64).copy()
        out["psi_k"] = np.frombuffer(read_record(f), np.float64).copy()
    p = os.path.join(outdir, "cont%02d.S2" % idproc)
    if os.path.exists(p):
        with open(p, "rb") as f:
            z = [np.frombuffer(read_record(f), np.complex128).copy() for _ in range(3)]
        out["zs2"] = z[0].reshape(zs2_shape) if zs2_shape else z[0]
        out["zcr"] = z[1].reshape(flux_shape) if flux_shape else z[1]
        out["zcdr"] = z[2].reshape(flux_shape) if flux_shape else z[2]
    p = os.path.join(outdir, "cont%02d.S2prod" % idproc)
    if os.path.exists(p):
        with open(p, "rb") as f:
            zp = np.frombuffer(read_record(f), np.complex128).copy()
        out["zs2prod"] = zp.reshape(prod_shape) if prod_shape else zp
    return out


def write_cvj_file(path, iterations, cvj):
    """Cvj.NNNN / Cvjprod.NNNN (SRC/main_madwave3.f:310-321, 354-364): one
    unformatted record per iteration holding the iteration number (4-byte
    integer) and the array (Cvj(nvini:nvmax, jini:jmax, ncan) or
    Cvjprod(nviniprod:nvmaxprod, jiniprod:jmaxprod, iomminprod:iommaxprod), the
    C order of mw3_download_cvj_history's rows)."""
    with open(path, "wb") as f:
        for it, row in zip(iterations, cvj):
            write_record(f, struct.pack("<i", int(it)) + np.ascontiguousarray(row, "<f8").tobytes())


def read_cvj_file(path, shape):
    """The (iterations, arrays [n][shape]) of a Cvj.NNNN / Cvjprod.NNNN file."""
    its, rows = [], []
    with open(path, "rb") as f:
        while True:
            try:
                b = read_record(f)
            except EOFError:
                break
            its.append(struct.unpack("<i", b[:4])[0])
            rows.append(np.frombuffer(b[4:], "<f8").reshape(shape))
    return np.array(its), np.array(rows)

