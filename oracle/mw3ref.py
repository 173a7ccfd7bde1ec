"""ctypes binding of the CPU oracle (oracle/mw3ref.c).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker.  The product path never imports
this module.
"""
import ctypes as ct
import os
import subprocess

import numpy as np

from madwave3_gb300.host import constants as C

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libmw3ref.so")

I32P = ct.POINTER(ct.c_int32)
F64P = ct.POINTER(ct.c_double)


class RefIn(ct.Structure):
    _fields_ = [
        ("npun1", ct.c_int32), ("npun2", ct.c_int32), ("nangu", ct.c_int32), ("nangu2", ct.c_int32),
        ("nelec", ct.c_int32), ("npun1min", ct.c_int32),
        ("rmis1", ct.c_double), ("rfin1", ct.c_double), ("ah1", ct.c_double),
        ("rmis2", ct.c_double), ("rfin2", ct.c_double), ("ah2", ct.c_double),
        ("hbr", ct.c_double), ("xm1red", ct.c_double), ("xm2red", ct.c_double),
        ("xm1reac", ct.c_double), ("xm2reac", ct.c_double),
        ("vcutmax", ct.c_double), ("radcutmax", ct.c_double), ("rotcutmax", ct.c_double),
        ("emindlt", ct.c_double), ("delta2", ct.c_double),
        ("proj_j2_up", ct.c_int32),
        ("npuntot", ct.c_int32),
        ("npunreal", I32P), ("indr1", I32P), ("indr2", I32P), ("vvv", F64P),
        ("Jtot", ct.c_int32), ("iparity", ct.c_int32), ("inc", ct.c_int32), ("j0", ct.c_int32),
        ("iommin", ct.c_int32), ("iommax", ct.c_int32), ("ncan", ct.c_int32),
        ("iombas", I32P), ("nelebas", I32P), ("nojbas", I32P), ("j00", I32P), ("jbas", I32P),
        ("iomdiat", I32P), ("iomatom", I32P), ("sigdiat", F64P), ("sigatom", F64P),
        ("djmmp", F64P),
        ("absr1", ct.c_double), ("absalp1", ct.c_double), ("absr2", ct.c_double), ("absalp2", ct.c_double),
        ("n1expo", ct.c_int32), ("ninterv1", ct.c_int32), ("n2expo", ct.c_int32), ("ninterv2", ct.c_int32),
        ("r1flux_ang", ct.c_double), ("ekinmin", ct.c_double), ("ekinmax", ct.c_double),
        ("netot", ct.c_int32), ("kminelastic", ct.c_int32), ("iphoto", ct.c_int32), ("iprod", ct.c_int32),
        ("nvini", ct.c_int32), ("nvmax", ct.c_int32), ("jini", ct.c_int32), ("jmax", ct.c_int32),
        ("nvref", ct.c_int32), ("jref", ct.c_int32), ("iomref", ct.c_int32), ("ielecref", ct.c_int32),
        ("nobc", I32P), ("ediat", F64P), ("fd", F64P),
        ("rcolini", ct.c_double), ("alpha0", ct.c_double), ("xk0", ct.c_double), ("factor0", ct.c_double),
        ("xmasa0", ct.c_double), ("il0", ct.c_int32),
        ("nofe", ct.c_int32), ("efe", F64P),
    ]


def build():
    """Compile the oracle with gcc (oracle/Makefile)."""
    subprocess.check_call(["make", "-s", "-C", HERE])


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ct.CDLL(LIB)
        L.mw3ref_create.restype = ct.c_void_p
        L.mw3ref_create.argtypes = [ct.POINTER(RefIn), ct.c_char_p, ct.c_int]
        L.mw3ref_destroy.argtypes = [ct.c_void_p]
        L.mw3ref_ntot.restype = ct.c_int64
        L.mw3ref_ntot.argtypes = [ct.c_void_p]
        L.mw3ref_set_threads.argtypes = [ct.c_void_p, ct.c_int]
        L.mw3ref_set_dst_mode.argtypes = [ct.c_void_p, ct.c_int]
        L.mw3ref_set_flux_gate.argtypes = [ct.c_void_p, ct.c_int]
        L.mw3ref_set_ecoriolis.argtypes = [ct.c_void_p, ct.c_int]
        L.mw3ref_autocorrelation.argtypes = [ct.c_void_p]
        L.mw3ref_autocorrelation.restype = ct.c_double
        for name in ("mw3ref_hphi",):
            getattr(L, name).argtypes = [ct.c_void_p, F64P, F64P]
        L.mw3ref_start.argtypes = [ct.c_void_p, F64P]
        L.mw3ref_run.argtypes = [ct.c_void_p, ct.c_int, F64P]
        L.mw3ref_get_state.argtypes = [ct.c_void_p, F64P, F64P, ct.POINTER(ct.c_int64)]
        L.mw3ref_set_state.argtypes = [ct.c_void_p, F64P, F64P, ct.c_int64]
        L.mw3ref_totalflux.argtypes = [ct.c_void_p, F64P, F64P]
        L.mw3ref_nflux.argtypes = [ct.c_void_p]
        L.mw3ref_get_flux.argtypes = [ct.c_void_p, F64P, F64P]
        L.mw3ref_get_s2.argtypes = [ct.c_void_p, F64P, F64P]
        L.mw3ref_get_zfe.argtypes = [ct.c_void_p, F64P]
        L.mw3ref_coefecheby.argtypes = [ct.c_void_p, ct.c_int64, F64P]
        L.mw3ref_tables.argtypes = [ct.c_void_p, I32P, F64P, F64P, F64P, F64P, I32P]
        L.mw3ref_flux_tables.argtypes = [ct.c_void_p, F64P, F64P, F64P, F64P, I32P]
        L.mw3ref_s2factor.argtypes = [ct.c_void_p, F64P]
        L.mw3ref_set_product.argtypes = [ct.c_void_p] + [ct.c_int] * 10 + [I32P, F64P, F64P, F64P]
        L.mw3ref_get_product.argtypes = [ct.c_void_p, F64P, F64P]
        L.mw3ref_xj2.argtypes = [ct.c_void_p, F64P]
        L.mw3ref_xl2p.argtypes = [ct.c_void_p, F64P]
        L.mw3ref_dst1.argtypes = [ct.c_int, F64P, F64P, ct.c_int]
        L.mw3ref_riccati.argtypes = [ct.c_int, ct.c_double, F64P, F64P]
        L.mw3ref_noptfft.argtypes = [ct.c_int, ct.c_int]
        L.mw3ref_sinmom_p2.argtypes = [ct.c_double, ct.c_int, ct.c_double, ct.c_double, F64P]
        L.mw3ref_absorption.argtypes = [ct.c_int, ct.c_double, ct.c_double, ct.c_double, ct.c_double, ct.c_int,
                                        ct.c_int, F64P, I32P]
        L.mw3ref_smatini_col.restype = ct.c_double
        L.mw3ref_smatini_col.argtypes = [ct.c_int] + [ct.c_double] * 10 + [ct.c_int, ct.c_double, F64P, F64P, F64P]
        _lib = L
    return _lib


def _p(a, typ):
    return a.ctypes.data_as(ct.POINTER(typ))


def dst1(x, mode=0):
    x = np.ascontiguousarray(x, np.float64)
    y = np.zeros_like(x)
    lib().mw3ref_dst1(len(x), _p(x, ct.c_double), _p(y, ct.c_double), mode)
    return y


def noptfft(nin, ntot):
    return lib().mw3ref_noptfft(nin, ntot)


def sinmom_p2(box, npun, xmred, hbr):
    out = np.zeros(npun)
    lib().mw3ref_sinmom_p2(box, npun, xmred, hbr, _p(out, ct.c_double))
    return out


def absorption(npun, rmis, ah, absr, absalp, nexpo, ninterv):
    f = np.zeros(npun)
    ir = ct.c_int32()
    lib().mw3ref_absorption(npun, rmis, ah, absr, absalp, nexpo, ninterv, _p(f, ct.c_double), ct.byref(ir))
    return f, ir.value


def smatini_col(netot, ekinmin, ekinmax, rmis2, rfin2, rcolini, xk0, alpha0, factor0, xmasa0, xm1reac, il0, hbr):
    et, ap, rf = np.zeros(netot), np.zeros(netot), np.zeros(netot)
    xn = lib().mw3ref_smatini_col(netot, ekinmin, ekinmax, rmis2, rfin2, rcolini, xk0, alpha0, factor0, xmasa0,
                                  xm1reac, il0, hbr, _p(et, ct.c_double), _p(ap, ct.c_double), _p(rf, ct.c_double))
    return xn, et, ap, rf


def riccati(l, x):
    f, g = ct.c_double(), ct.c_double()
    lib().mw3ref_riccati(l, x, ct.byref(f), ct.byref(g))
    return f.value, g.value


class Oracle:
    """One partial wave on the CPU oracle, built from a host ``setup.Run``."""

    def __init__(self, run, nofe_energies_ev=None, threads=1, dst_mode=0, flux_gate=True, ecoriolis=False):
        i = run.inp
        self.run = run
        keep = {}

        def arr(name, a, dt):
            a = np.ascontiguousarray(a, dt)
            keep[name] = a
            return _p(a, ct.c_int32 if dt == np.int32 else ct.c_double)

        s = RefIn()
        s.npun1, s.npun2, s.nangu, s.nangu2 = i.npun1, i.npun2, i.nangu, run.nangu2
        s.nelec, s.npun1min = run.nelec, i.npun1min
        s.rmis1, s.rfin1, s.ah1 = i.rmis1, i.rfin1, run.ah1
        s.rmis2, s.rfin2, s.ah2 = i.rmis2, i.rfin2, run.ah2
        s.hbr, s.xm1red, s.xm2red, s.xm1reac, s.xm2reac = C.hbr, run.xm1red, run.xm2red, run.xm1reac, run.xm2reac
        s.vcutmax, s.radcutmax, s.rotcutmax = run.vcutmax, run.radcutmax, run.rotcutmax
        s.emindlt, s.delta2 = run.emindlt, run.delta2
        s.proj_j2_up = i.proj_j2_up
        s.npuntot = run.npuntot
        s.npunreal = arr("npunreal", run.npunreal, np.int32)
        s.indr1 = arr("indr1", run.indr1, np.int32)
        s.indr2 = arr("indr2", run.indr2, np.int32)
        s.vvv = arr("vvv", run.vvv, np.float64)
        s.Jtot, s.iparity, s.inc, s.j0 = i.Jtot, i.iparity, i.inc, i.j0
        s.iommin, s.iommax, s.ncan = i.iommin, i.iommax, run.ncan
        s.iombas = arr("iombas", run.iombas, np.int32)
        s.nelebas = arr("nelebas", run.nelebas, np.int32)
        s.nojbas = arr("nojbas", run.nojbas, np.int32)
        s.j00 = arr("j00", run.j00, np.int32)
        s.jbas = arr("jbas", run.jbas, np.int32)
        s.iomdiat = arr("iomdiat", run.iomdiat, np.int32)
        s.iomatom = arr("iomatom", run.iomatom, np.int32)
        s.sigdiat = arr("sigdiat", run.sigdiat, np.float64)
        s.sigatom = arr("sigatom", run.sigatom, np.float64)
        s.djmmp = arr("djmmp", run.djmmp, np.float64)
        s.absr1, s.absalp1, s.absr2, s.absalp2 = i.absr1, i.absalp1, i.absr2, i.absalp2
        s.n1expo, s.ninterv1, s.n2expo, s.ninterv2 = i.n1expo, i.ninterv1, i.n2expo, i.ninterv2
        s.r1flux_ang = i.r1flux_ang
        s.ekinmin = i.ekinmin_ev * C.eV2cm * C.conve1
        s.ekinmax = i.ekinmax_ev * C.eV2cm * C.conve1
        s.netot, s.kminelastic, s.iphoto, s.iprod = i.netot, i.kminelastic, i.iphoto, i.iprod
        s.nvini, s.nvmax, s.jini, s.jmax = i.nvini, i.nvmax, i.jini, i.jmax
        s.nvref, s.jref, s.iomref, s.ielecref = i.nvref, i.jref, i.iomref, i.ielecref
        s.nobc = arr("nobc", run.nobc, np.int32)
        s.ediat = arr("ediat", run.ediat, np.float64)
        s.fd = arr("fd", run.fd, np.float64)
        s.rcolini, s.alpha0, s.xk0, s.factor0 = run.rcolini, run.alpha0, run.xk0, run.factor0
        s.xmasa0, s.il0 = run.xmasa0, run.il0
        efe = np.array([e * C.eV2cm * C.conve1 for e in (nofe_energies_ev or [])], np.float64)
        s.nofe = len(efe)
        s.efe = arr("efe", efe if len(efe) else np.zeros(1), np.float64)
        self._keep = keep
        self._s = s
        err = ct.create_string_buffer(512)
        h = lib().mw3ref_create(ct.byref(s), err, 512)
        if not h:
            raise RuntimeError("mw3ref_create: " + err.value.decode())
        self.h = h
        self.ntot = lib().mw3ref_ntot(h)
        lib().mw3ref_set_threads(h, threads)
        lib().mw3ref_set_dst_mode(h, dst_mode)
        lib().mw3ref_set_flux_gate(h, 1 if flux_gate else 0)
        if ecoriolis:
            lib().mw3ref_set_ecoriolis(h, 1)
        self.netot = i.netot
        self.nelec = run.nelec
        self.nj = i.jmax - i.jini + 1
        self.nv = i.nvmax - i.nvini + 1
        self.nofe = s.nofe

    def __del__(self):
        if getattr(self, "h", None):
            lib().mw3ref_destroy(self.h)
            self.h = None

    def set_threads(self, n):
        lib().mw3ref_set_threads(self.h, n)

    def hphi(self, psi):
        psi = np.ascontiguousarray(psi, np.float64)
        out = np.zeros(self.ntot)
        lib().mw3ref_hphi(self.h, _p(psi, ct.c_double), _p(out, ct.c_double))
        return out

    def start(self, psi0):
        psi0 = np.ascontiguousarray(psi0, np.float64)
        lib().mw3ref_start(self.h, _p(psi0, ct.c_double))

    def run_iters(self, n):
        norms = np.zeros(n)
        lib().mw3ref_run(self.h, n, _p(norms, ct.c_double))
        return norms

    def run_autocorrelation(self, n):
        """n iterations one by one: (norms, <psi0|psi_k>) after each (iphoto >= 1)."""
        norms, autos = np.zeros(n), np.zeros(n)
        for k in range(n):
            norms[k] = self.run_iters(1)[0]
            autos[k] = lib().mw3ref_autocorrelation(self.h)
        return norms, autos

    def state(self):
        a, b = np.zeros(self.ntot), np.zeros(self.ntot)
        it = ct.c_int64()
        lib().mw3ref_get_state(self.h, _p(a, ct.c_double), _p(b, ct.c_double), ct.byref(it))
        return a, b, it.value

    def set_state(self, km1, k, it):
        km1 = np.ascontiguousarray(km1, np.float64)
        k = np.ascontiguousarray(k, np.float64)
        lib().mw3ref_set_state(self.h, _p(km1, ct.c_double), _p(k, ct.c_double), it)

    def totalflux(self):
        tot = np.zeros(self.netot)
        el = np.zeros((self.nelec, self.netot))
        lib().mw3ref_totalflux(self.h, _p(tot, ct.c_double), _p(el, ct.c_double))
        return tot, el

    def nflux(self):
        return lib().mw3ref_nflux(self.h)

    def flux(self):
        nf = self.nflux()
        a = np.zeros((nf, self.netot, 2))
        b = np.zeros((nf, self.netot, 2))
        lib().mw3ref_get_flux(self.h, _p(a, ct.c_double), _p(b, ct.c_double))
        return a[..., 0] + 1j * a[..., 1], b[..., 0] + 1j * b[..., 1]

    def s2(self):
        nc = self.run.ncan
        z = np.zeros((nc, self.nj, self.nv, self.netot, 2))
        c = np.zeros((nc, self.nj, self.nv))
        lib().mw3ref_get_s2(self.h, _p(z, ct.c_double), _p(c, ct.c_double))
        return z[..., 0] + 1j * z[..., 1], c

    def zfe(self):
        z = np.zeros((self.nofe, self.ntot, 2))
        lib().mw3ref_get_zfe(self.h, _p(z, ct.c_double))
        return z[..., 0] + 1j * z[..., 1]

    def coefecheby(self, k):
        ck = np.zeros((self.netot, 2))
        lib().mw3ref_coefecheby(self.h, k, _p(ck, ct.c_double))
        return ck[:, 0] + 1j * ck[:, 1]

    def tables(self):
        run = self.run
        i = run.inp
        nopr1 = np.zeros(i.nangu, np.int32)
        p2r1 = np.zeros((i.nangu, i.npun1))
        p2r2 = np.zeros((i.nangu, i.npun2))
        a1, a2 = np.zeros(i.npun1), np.zeros(i.npun2)
        irabs = np.zeros(2, np.int32)
        lib().mw3ref_tables(self.h, _p(nopr1, ct.c_int32), _p(p2r1, ct.c_double), _p(p2r2, ct.c_double),
                            _p(a1, ct.c_double), _p(a2, ct.c_double), _p(irabs, ct.c_int32))
        return dict(nopr1=nopr1, p2r1=p2r1, p2r2=p2r2, absfr1=a1, absfr2=a2,
                    ir1abs=int(irabs[0]), ir2abs=int(irabs[1]))

    def flux_tables(self):
        n = self.netot
        et, rf, ap = np.zeros(n), np.zeros(n), np.zeros(n)
        za = np.zeros((self.run.inp.npun1, 2))
        ir4 = ct.c_int32()
        lib().mw3ref_flux_tables(self.h, _p(et, ct.c_double), _p(rf, ct.c_double), _p(ap, ct.c_double),
                                 _p(za, ct.c_double), ct.byref(ir4))
        return dict(etot=et, reacfct=rf, apaqini=ap, zar1flux=za[:, 0] + 1j * za[:, 1], ir4flux=ir4.value)

    def set_product(self, pp):
        """pp: ProductProjection (madwave3_gb300.product) with the tables of
        ini_transcoor; the run then does prodpaq and prodcvj every iteration."""
        self._prod = (np.ascontiguousarray(pp.nobcprod, np.int32), np.ascontiguousarray(pp.transrgjac, np.float64),
                      np.ascontiguousarray(pp.dtrans, np.float64), np.ascontiguousarray(pp.prodwf, np.float64))
        rc = lib().mw3ref_set_product(self.h, pp.n2prod0, pp.n2prod1, pp.nangproj0, pp.nangproj1, pp.iomminprod,
                                      pp.iommaxprod, pp.jiniprod, pp.jmaxprod, pp.nviniprod, pp.nvmaxprod,
                                      _p(self._prod[0], ct.c_int32), _p(self._prod[1], ct.c_double),
                                      _p(self._prod[2], ct.c_double), _p(self._prod[3], ct.c_double))
        if rc:
            raise ValueError("bad product projection ranges")
        self._prodshape = (pp.iommaxprod - pp.iomminprod + 1, pp.jmaxprod - pp.jiniprod + 1,
                           pp.nvmaxprod - pp.nviniprod + 1)

    def product(self):
        z = np.zeros(self._prodshape + (self.netot, 2))
        c = np.zeros(self._prodshape)
        lib().mw3ref_get_product(self.h, _p(z, ct.c_double), _p(c, ct.c_double))
        return z[..., 0] + 1j * z[..., 1], c

    def s2factor(self):
        out = np.zeros((self.run.nelec, self.nj, self.nv, self.netot))
        lib().mw3ref_s2factor(self.h, _p(out, ct.c_double))
        return out

    def xj2(self):
        r = self.run
        a = np.zeros((r.ncan, r.inp.nangu, r.inp.nangu, r.inp.npun1))
        lib().mw3ref_xj2(self.h, _p(a, ct.c_double))
        return a

    def xl2p(self):
        r = self.run
        a = np.zeros((3, r.ncan, r.inp.nangu, r.inp.nangu, r.inp.npun2))
        lib().mw3ref_xl2p(self.h, _p(a, ct.c_double))
        return a
