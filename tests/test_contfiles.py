"""Continuation files (wvpcont, SRC/main_madwave3.f:496-551): gfortran's
unformatted sequential framing, subrecords, and the four files' round trip."""
import io
import struct

import numpy as np

from madwave3_gb300 import contfiles


def test_record_framing():
    f = io.BytesIO()
    a = np.arange(3, dtype=np.float64)
    contfiles.write_record(f, a)
    b = f.getvalue()
    assert len(b) == 4 + 24 + 4
    assert struct.unpack("<i", b[:4])[0] == 24 and struct.unpack("<i", b[-4:])[0] == 24
    assert np.array_equal(np.frombuffer(b[4:-4], np.float64), a)


def test_subrecords():
    """A record longer than a subrecord: leading count negative while the record
    continues, trailing count negative after the first piece."""
    f = io.BytesIO()
    data = bytes(range(250)) * 2
    contfiles.write_record(f, data, max_sub=200)
    contfiles.write_record(f, b"tail", max_sub=200)
    b = f.getvalue()
    heads = []
    pos = 0
    for _ in range(3):
        L = struct.unpack("<i", b[pos:pos + 4])[0]
        T = struct.unpack("<i", b[pos + 4 + abs(L):pos + 8 + abs(L)])[0]
        heads.append((L, T))
        pos += 8 + abs(L)
    assert heads == [(-200, 200), (-200, -200), (100, -100)]
    f.seek(0)
    assert contfiles.read_record(f) == data
    assert contfiles.read_record(f) == b"tail"


def test_cont_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    km1, k = rng.standard_normal(50), rng.standard_normal(50)
    zs2 = rng.standard_normal((2, 3, 2, 7)) + 1j * rng.standard_normal((2, 3, 2, 7))
    zcr = rng.standard_normal((5, 7)) + 1j * rng.standard_normal((5, 7))
    zcdr = rng.standard_normal((5, 7)) + 1j * rng.standard_normal((5, 7))
    zp = rng.standard_normal((1, 2, 2, 7)) + 1j * rng.standard_normal((1, 2, 2, 7))
    contfiles.write_cont(str(tmp_path), km1, k, zs2, zcr, zcdr, iit0=1500, indt=2, iloop=3, abstot=0.25,
                         zs2prod=zp)
    r = contfiles.read_cont(str(tmp_path), zs2_shape=zs2.shape, flux_shape=zcr.shape, prod_shape=zp.shape)
    assert (r["iit0"], r["indt"], r["iloop"], r["nflux"], r["ncan"]) == (1500, 3, 3, 5, 2)
    for key, v in (("psi_km1", km1), ("psi_k", k), ("zs2", zs2), ("zcr", zcr), ("zcdr", zcdr), ("zs2prod", zp)):
        assert np.array_equal(r[key], v), key
    # complex*16 is (re, im) pairs: the same bytes as the library's interleaved arrays
    with open(tmp_path / "cont00.S2", "rb") as f:
        raw = np.frombuffer(contfiles.read_record(f), np.float64)
    assert np.array_equal(raw[0::2], zs2.real.ravel()) and np.array_equal(raw[1::2], zs2.imag.ravel())
