"""Python host side over the C-ABI of libmw3gpu (include/mw3gpu.h).

Mirrors the reference's module interface for the hot path: ``difs`` becomes
:meth:`Propagator.hphi`, the time loop of main_madwave3.f (:308-368) becomes
:meth:`Propagator.start` + :meth:`Propagator.run`, ``totalflux`` becomes
:meth:`Propagator.totalflux`, and the accumulators ``zCR``/``zCdR``/``zS2``/
``Cvj``/``zfE`` are read back with :meth:`Propagator.accumulators`.  Error
behaviour follows the reference's convention of stopping on bad input: every
non-zero status raises :class:`Mw3Error` with the library's message.

The compute path is the CUDA library only; there is no CPU fallback.  Loading
fails loudly when the library is missing or no CUDA device is present.
"""
import ctypes as ct
import os

import numpy as np

from .host import constants as C

I32P = ct.POINTER(ct.c_int32)
F64P = ct.POINTER(ct.c_double)

PREC_FP64 = 0
PREC_MIXED = 1


class Mw3Error(RuntimeError):
    pass


class Grid(ct.Structure):
    _fields_ = [
        ("npun1", ct.c_int32), ("npun2", ct.c_int32), ("nangu", ct.c_int32), ("nelec", ct.c_int32),
        ("npun1min", ct.c_int32), ("npuntot", ct.c_int32),
        ("rmis1", ct.c_double), ("rfin1", ct.c_double), ("rmis2", ct.c_double), ("rfin2", ct.c_double),
        ("hbr", ct.c_double), ("xm1red", ct.c_double), ("xm2red", ct.c_double),
        ("radcutmax", ct.c_double), ("rotcutmax", ct.c_double),
        ("emindlt", ct.c_double), ("delta2", ct.c_double),
        ("precision", ct.c_int32),
    ]


class Wave(ct.Structure):
    _fields_ = [
        ("Jtot", ct.c_int32), ("iparity", ct.c_int32), ("inc", ct.c_int32), ("j0", ct.c_int32),
        ("iommin", ct.c_int32), ("iommax", ct.c_int32), ("ncan", ct.c_int32),
        ("iombas", I32P), ("nelebas", I32P), ("nojbas", I32P), ("j00", I32P), ("jbas", I32P),
        ("iomdiat", I32P), ("iomatom", I32P), ("sigdiat", F64P), ("sigatom", F64P),
        ("nangu2", ct.c_int32), ("djmmp", F64P), ("proj_j2_up", ct.c_int32),
        ("absr1", ct.c_double), ("absalp1", ct.c_double), ("absr2", ct.c_double), ("absalp2", ct.c_double),
        ("n1expo", ct.c_int32), ("ninterv1", ct.c_int32), ("n2expo", ct.c_int32), ("ninterv2", ct.c_int32),
        ("r1flux_ang", ct.c_double), ("ekinmin", ct.c_double), ("ekinmax", ct.c_double),
        ("netot", ct.c_int32), ("kminelastic", ct.c_int32), ("iphoto", ct.c_int32), ("iprod", ct.c_int32),
        ("nvini", ct.c_int32), ("nvmax", ct.c_int32), ("jini", ct.c_int32), ("jmax", ct.c_int32),
        ("nvref", ct.c_int32), ("jref", ct.c_int32), ("iomref", ct.c_int32), ("ielecref", ct.c_int32),
        ("nobc", I32P), ("ediat", F64P), ("fd", F64P),
        ("xm1reac", ct.c_double), ("xm2reac", ct.c_double),
        ("rcolini", ct.c_double), ("alpha0", ct.c_double), ("xk0", ct.c_double), ("factor0", ct.c_double),
        ("xmasa0", ct.c_double), ("il0", ct.c_int32),
        ("nofe", ct.c_int32), ("efe", F64P),
    ]


HEADER_FUNCS = [
    "mw3_create", "mw3_add_wave", "mw3_wave_size", "mw3_hphi", "mw3_start", "mw3_upload_state",
    "mw3_run", "mw3_sync", "mw3_download_state", "mw3_upload_state_all", "mw3_download_state_all",
    "mw3_norms", "mw3_totalflux", "mw3_flux_count",
    "mw3_download_accumulators", "mw3_tables", "mw3_packet_energy_norm", "mw3_kernel_launches", "mw3_path_flags",
    "mw3_get_stream",
    "mw3_profile",
    "mw3_stage_times", "mw3_hphi_noalloc", "mw3_set_product_projection", "mw3_download_product",
    "mw3_cvj_history", "mw3_download_cvj_history", "mw3_set_flux_gate", "mw3_set_ecoriolis", "mw3_set_choices",
    "mw3_get_choices", "mw3_autotune", "mw3_autocorrelation",
    "mw3_upload_accumulators", "mw3_upload_product",
    "mw3_last_error", "mw3_destroy",
]
# stage 0 holds the whole radial DST chain when the mixed path runs it as one
# fused kernel (stages 1 and 2 are then empty); stage 3 is the whole angular
# part when it runs as one fused tensor-core contraction (stage 4 then empty)
STAGES = ["dst_R", "dst_r_pair", "dst_R_gather", "angular", "angular_l2", "update", "accumulators"]

_lib = None


def library_path():
    from . import build as _b
    return _b.LIB


def load_library(build_if_missing=True):
    """Load libmw3gpu.so from the package's build folder (building it if asked)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise Mw3Error("libmw3gpu.so is not built (run madwave3_gb300.build.build())")
        from . import build as _b
        _b.build()
    L = ct.CDLL(path)
    vp = ct.c_void_p
    L.mw3_create.argtypes = [ct.POINTER(vp), ct.POINTER(Grid), I32P, I32P, I32P, F64P]
    L.mw3_add_wave.argtypes = [vp, ct.POINTER(Wave), I32P]
    L.mw3_wave_size.argtypes = [vp, ct.c_int32, ct.POINTER(ct.c_int64)]
    L.mw3_hphi.argtypes = [vp, ct.c_int32, F64P, F64P]
    L.mw3_start.argtypes = [vp, ct.POINTER(F64P)]
    L.mw3_upload_state.argtypes = [vp, ct.c_int32, F64P, F64P, ct.c_int64]
    L.mw3_run.argtypes = [vp, ct.c_int64]
    L.mw3_sync.argtypes = [vp]
    L.mw3_download_state.argtypes = [vp, ct.c_int32, F64P, F64P, ct.POINTER(ct.c_int64)]
    L.mw3_upload_state_all.argtypes = [vp, F64P, F64P, ct.c_int64]
    L.mw3_download_state_all.argtypes = [vp, F64P, F64P, ct.POINTER(ct.c_int64)]
    L.mw3_norms.argtypes = [vp, ct.c_int32, F64P, ct.POINTER(ct.c_int64)]
    L.mw3_totalflux.argtypes = [vp, ct.c_int32, F64P, F64P]
    L.mw3_flux_count.argtypes = [vp, ct.c_int32, I32P]
    L.mw3_download_accumulators.argtypes = [vp, ct.c_int32, F64P, F64P, F64P, F64P, F64P]
    L.mw3_tables.argtypes = [vp, ct.c_int32, I32P, F64P, F64P, F64P, F64P, F64P]
    L.mw3_packet_energy_norm.argtypes = [vp, ct.c_int32, F64P]
    L.mw3_cvj_history.argtypes = [vp, ct.c_int64]
    L.mw3_autocorrelation.argtypes = [vp, ct.c_int32, F64P, ct.POINTER(ct.c_int64)]
    L.mw3_set_flux_gate.argtypes = [vp, ct.c_int32, ct.c_int32]
    L.mw3_set_ecoriolis.argtypes = [vp, ct.c_int32, ct.c_int32]
    L.mw3_set_choices.argtypes = [vp, ct.POINTER(ct.c_int32)]
    L.mw3_get_choices.argtypes = [vp, ct.POINTER(ct.c_int32)]
    L.mw3_autotune.argtypes = [vp, ct.c_int32, ct.c_int32, ct.POINTER(ct.c_int32), ct.POINTER(ct.c_double)]
    L.mw3_download_cvj_history.argtypes = [vp, ct.c_int32, ct.c_int64, F64P, F64P, ct.POINTER(ct.c_int64)]
    L.mw3_kernel_launches.argtypes = [vp, ct.POINTER(ct.c_int64)]
    L.mw3_path_flags.argtypes = [vp, ct.POINTER(ct.c_int32)]
    L.mw3_get_stream.argtypes = [vp, ct.POINTER(ct.c_void_p)]
    L.mw3_profile.argtypes = [vp, ct.c_int]
    L.mw3_stage_times.argtypes = [vp, F64P, ct.POINTER(ct.c_int64)]
    L.mw3_set_product_projection.argtypes = [vp, ct.c_int32, ct.POINTER(ProdProj)]
    L.mw3_download_product.argtypes = [vp, ct.c_int32, F64P, F64P]
    L.mw3_upload_accumulators.argtypes = [vp, ct.c_int32, F64P, F64P, F64P]
    L.mw3_upload_product.argtypes = [vp, ct.c_int32, F64P]
    L.mw3_last_error.argtypes = [vp]
    L.mw3_last_error.restype = ct.c_char_p
    L.mw3_destroy.argtypes = [vp]
    _lib = L
    return L


def _p(a, typ=ct.c_double):
    return a.ctypes.data_as(ct.POINTER(typ))


class ProdProj(ct.Structure):
    """mw3_prodproj"""
    _fields_ = [(n, ct.c_int32) for n in ("n2prod0", "n2prod1", "nangproj0", "nangproj1", "iomminprod",
                                          "iommaxprod", "jiniprod", "jmaxprod", "nviniprod", "nvmaxprod")] + \
               [("nobcprod", I32P), ("transrgjac", F64P), ("dtrans", F64P), ("prodwf", F64P)]


class Propagator:
    """Every partial wave of a batch, propagated together on one GPU.

    ``runs`` are host set-ups (:func:`madwave3_gb300.host.setup.load`) that
    share one grid and potential; ``precision`` is "fp64" (the reference's
    arithmetic) or "mixed" (FP32 transforms, FP64 recursion/accumulators).
    """

    def __init__(self, runs, precision="fp64"):
        if not isinstance(runs, (list, tuple)):
            runs = [runs]
        self.L = load_library()
        self.runs = list(runs)
        r0 = runs[0]
        i = r0.inp
        self._keep = []
        g = Grid()
        g.npun1, g.npun2, g.nangu, g.nelec = i.npun1, i.npun2, i.nangu, r0.nelec
        g.npun1min, g.npuntot = i.npun1min, r0.npuntot
        g.rmis1, g.rfin1, g.rmis2, g.rfin2 = i.rmis1, i.rfin1, i.rmis2, i.rfin2
        g.hbr, g.xm1red, g.xm2red = C.hbr, r0.xm1red, r0.xm2red
        g.radcutmax, g.rotcutmax = r0.radcutmax, r0.rotcutmax
        g.emindlt, g.delta2 = r0.emindlt, r0.delta2
        g.precision = PREC_FP64 if precision == "fp64" else PREC_MIXED
        self.precision = precision
        npunreal = self._k(r0.npunreal, np.int32)
        indr1 = self._k(r0.indr1, np.int32)
        indr2 = self._k(r0.indr2, np.int32)
        vvv = self._k(r0.vvv, np.float64)
        h = ct.c_void_p()
        rc = self.L.mw3_create(ct.byref(h), ct.byref(g), _p(npunreal, ct.c_int32), _p(indr1, ct.c_int32),
                               _p(indr2, ct.c_int32), _p(vvv))
        if rc != 0:
            raise Mw3Error("mw3_create failed with status %d" % rc)
        self.h = h
        self.ntot = []
        for r in self.runs:
            self._add_wave(r)

    def _k(self, a, dt):
        a = np.ascontiguousarray(a, dt)
        self._keep.append(a)
        return a

    def _check(self, rc, what):
        if rc != 0:
            msg = self.L.mw3_last_error(self.h)
            raise Mw3Error("%s failed with status %d: %s" % (what, rc, msg.decode() if msg else ""))

    def _add_wave(self, r):
        i = r.inp
        w = Wave()
        w.Jtot, w.iparity, w.inc, w.j0 = i.Jtot, i.iparity, i.inc, i.j0
        w.iommin, w.iommax, w.ncan = i.iommin, i.iommax, r.ncan
        w.iombas = _p(self._k(r.iombas, np.int32), ct.c_int32)
        w.nelebas = _p(self._k(r.nelebas, np.int32), ct.c_int32)
        w.nojbas = _p(self._k(r.nojbas, np.int32), ct.c_int32)
        w.j00 = _p(self._k(r.j00, np.int32), ct.c_int32)
        w.jbas = _p(self._k(r.jbas, np.int32), ct.c_int32)
        w.iomdiat = _p(self._k(r.iomdiat, np.int32), ct.c_int32)
        w.iomatom = _p(self._k(r.iomatom, np.int32), ct.c_int32)
        w.sigdiat = _p(self._k(r.sigdiat, np.float64))
        w.sigatom = _p(self._k(r.sigatom, np.float64))
        w.nangu2 = r.nangu2
        w.djmmp = _p(self._k(r.djmmp, np.float64))
        w.proj_j2_up = i.proj_j2_up
        w.absr1, w.absalp1, w.absr2, w.absalp2 = i.absr1, i.absalp1, i.absr2, i.absalp2
        w.n1expo, w.ninterv1, w.n2expo, w.ninterv2 = i.n1expo, i.ninterv1, i.n2expo, i.ninterv2
        w.r1flux_ang = i.r1flux_ang
        w.ekinmin = i.ekinmin_ev * C.eV2cm * C.conve1
        w.ekinmax = i.ekinmax_ev * C.eV2cm * C.conve1
        w.netot, w.kminelastic, w.iphoto, w.iprod = i.netot, i.kminelastic, i.iphoto, i.iprod
        w.nvini, w.nvmax, w.jini, w.jmax = i.nvini, i.nvmax, i.jini, i.jmax
        w.nvref, w.jref, w.iomref, w.ielecref = i.nvref, i.jref, i.iomref, i.ielecref
        w.nobc = _p(self._k(r.nobc, np.int32), ct.c_int32)
        w.ediat = _p(self._k(r.ediat, np.float64))
        w.fd = _p(self._k(r.fd, np.float64))
        w.xm1reac, w.xm2reac = r.xm1reac, r.xm2reac
        w.rcolini, w.alpha0, w.xk0, w.factor0 = r.rcolini, r.alpha0, r.xk0, r.factor0
        w.xmasa0, w.il0 = r.xmasa0, r.il0
        efe = getattr(r, "efe_zot", None)
        if efe is not None and len(efe):
            w.nofe = len(efe)
            w.efe = _p(self._k(np.asarray(efe, np.float64), np.float64))
        else:
            w.nofe = 0
            w.efe = _p(self._k(np.zeros(1), np.float64))
        wid = ct.c_int32()
        self._check(self.L.mw3_add_wave(self.h, ct.byref(w), ct.byref(wid)), "mw3_add_wave")
        n = ct.c_int64()
        self._check(self.L.mw3_wave_size(self.h, wid.value, ct.byref(n)), "mw3_wave_size")
        if n.value != r.ntot:
            raise Mw3Error("wave size mismatch: library %d, host %d" % (n.value, r.ntot))
        self.ntot.append(n.value)

    # ---- the reference's operations -------------------------------------
    def hphi(self, psi, wave=0):
        """difs: H psi for one wave (host arrays in and out)."""
        psi = np.ascontiguousarray(psi, np.float64)
        out = np.empty(self.ntot[wave])
        self._check(self.L.mw3_hphi(self.h, wave, _p(psi), _p(out)), "mw3_hphi")
        return out

    def start(self, psi0s=None):
        """Fresh start from each wave's initial packet (default: the host's psi0)."""
        if psi0s is None:
            psi0s = [r.psi0 for r in self.runs]
        arrs = [np.ascontiguousarray(p, np.float64) for p in psi0s]
        ptrs = (F64P * len(arrs))(*[_p(a) for a in arrs])
        self._check(self.L.mw3_start(self.h, ptrs), "mw3_start")

    def set_product_projection(self, pp, wave=0):
        """prodpaq / prodcvj every iteration for this wave (iprod = 2); pp is a
        madwave3_gb300.product.ProductProjection.  Before the first hphi/start."""
        keep = (np.ascontiguousarray(pp.nobcprod, np.int32), np.ascontiguousarray(pp.transrgjac, np.float64),
                np.ascontiguousarray(pp.dtrans, np.float64), np.ascontiguousarray(pp.prodwf, np.float64))
        s = ProdProj(pp.n2prod0, pp.n2prod1, pp.nangproj0, pp.nangproj1, pp.iomminprod, pp.iommaxprod,
                     pp.jiniprod, pp.jmaxprod, pp.nviniprod, pp.nvmaxprod, _p(keep[0], ct.c_int32), _p(keep[1]),
                     _p(keep[2]), _p(keep[3]))
        self._check(self.L.mw3_set_product_projection(self.h, wave, ct.byref(s)), "mw3_set_product_projection")
        if not hasattr(self, "_prodshape"):
            self._prodshape = {}
        self._prodshape[wave] = pp.shape

    def product(self, wave=0):
        """(zS2prod [nom][njp][nvp][netot] complex, last Cvjprod [nom][njp][nvp])."""
        shp = self._prodshape[wave]
        z = np.empty(shp + (self.runs[wave].inp.netot, 2))
        c = np.empty(shp)
        self._check(self.L.mw3_download_product(self.h, wave, _p(z), _p(c)), "mw3_download_product")
        return z[..., 0] + 1j * z[..., 1], c

    def upload_accumulators(self, wave, zcr, zcdr, zs2):
        """A restart's zCR, zCdR, zS2 (complex arrays as .accumulators() returns)."""
        arr = [None if a is None else np.ascontiguousarray(np.stack([np.real(a), np.imag(a)], -1), np.float64)
               for a in (zcr, zcdr, zs2)]
        ptr = [None if a is None else _p(a) for a in arr]
        self._check(self.L.mw3_upload_accumulators(self.h, wave, *ptr), "mw3_upload_accumulators")

    def upload_product(self, zs2prod, wave=0):
        a = np.ascontiguousarray(np.stack([np.real(zs2prod), np.imag(zs2prod)], -1), np.float64)
        self._check(self.L.mw3_upload_product(self.h, wave, _p(a)), "mw3_upload_product")

    def upload_state(self, wave, psi_km1, psi_k, it):
        a = np.ascontiguousarray(psi_km1, np.float64)
        b = np.ascontiguousarray(psi_k, np.float64)
        self._check(self.L.mw3_upload_state(self.h, wave, _p(a), _p(b), it), "mw3_upload_state")

    def upload_state_all(self, psi_km1, psi_k, it):
        """Every wave's state at once: the vectors back to back in wave order.
        psi_km1 None keeps the device's psi_k-1 (only psi_k is replaced)."""
        b = np.ascontiguousarray(psi_k, np.float64)
        assert b.size == sum(self.ntot)
        if psi_km1 is None:
            pa = None
        else:
            a = np.ascontiguousarray(psi_km1, np.float64)
            assert a.size == b.size
            pa = _p(a)
        self._check(self.L.mw3_upload_state_all(self.h, pa, _p(b), it), "mw3_upload_state_all")

    def state_all(self, out_km1=None, out_k=None):
        """Every wave's state at once, back to back in wave order."""
        n = sum(self.ntot)
        a = np.empty(n) if out_km1 is None else out_km1
        b = np.empty(n) if out_k is None else out_k
        assert a.size == b.size == n and a.dtype == b.dtype == np.float64
        it = ct.c_int64()
        self._check(self.L.mw3_download_state_all(self.h, _p(a), _p(b), ct.byref(it)), "mw3_download_state_all")
        return a, b, it.value

    def state_k_all(self, out_k):
        """psi_k of every wave (back to back in wave order) into out_k."""
        assert out_k.size == sum(self.ntot) and out_k.dtype == np.float64
        it = ct.c_int64()
        self._check(self.L.mw3_download_state_all(self.h, None, _p(out_k), ct.byref(it)), "mw3_download_state_all")
        return it.value

    def run(self, n):
        self._check(self.L.mw3_run(self.h, n), "mw3_run")

    def sync(self):
        self._check(self.L.mw3_sync(self.h), "mw3_sync")

    def state(self, wave=0, out_km1=None, out_k=None):
        a = np.empty(self.ntot[wave]) if out_km1 is None else out_km1
        b = np.empty(self.ntot[wave]) if out_k is None else out_k
        it = ct.c_int64()
        self._check(self.L.mw3_download_state(self.h, wave, _p(a), _p(b), ct.byref(it)), "mw3_download_state")
        return a, b, it.value

    def norms(self, wave=0, cap=1 << 22):
        buf = np.empty(cap)
        n = ct.c_int64(cap)
        self._check(self.L.mw3_norms(self.h, wave, _p(buf), ct.byref(n)), "mw3_norms")
        return buf[: n.value].copy()

    def autocorrelation(self, wave=0, cap=1 << 22):
        """<psi0|psi_k>, k = 1, 2, ... of a photodissociation wave (check)."""
        buf = np.empty(cap)
        n = ct.c_int64(cap)
        self._check(self.L.mw3_autocorrelation(self.h, wave, _p(buf), ct.byref(n)), "mw3_autocorrelation")
        return buf[: n.value].copy()

    def totalflux(self, wave=0):
        r = self.runs[wave]
        netot = r.inp.netot
        tot = np.empty(netot)
        el = np.empty((r.nelec, netot))
        self._check(self.L.mw3_totalflux(self.h, wave, _p(tot), _p(el)), "mw3_totalflux")
        return tot, el

    def nflux(self, wave=0):
        n = ct.c_int32()
        self._check(self.L.mw3_flux_count(self.h, wave, ct.byref(n)), "mw3_flux_count")
        return n.value

    def accumulators(self, wave=0):
        r = self.runs[wave]
        i = r.inp
        netot = i.netot
        nj, nv = i.jmax - i.jini + 1, i.nvmax - i.nvini + 1
        nf = self.nflux(wave)
        zcr = np.empty((nf, netot, 2))
        zcdr = np.empty((nf, netot, 2))
        zs2 = np.empty((r.ncan, nj, nv, netot, 2))
        cvj = np.empty((r.ncan, nj, nv))
        self._check(self.L.mw3_download_accumulators(self.h, wave, _p(zcr), _p(zcdr), _p(zs2), _p(cvj), None),
                    "mw3_download_accumulators")
        cx = lambda a: a[..., 0] + 1j * a[..., 1]
        return dict(zcr=cx(zcr), zcdr=cx(zcdr), zs2=cx(zs2), cvj=cvj)

    def set_flux_gate(self, on, wave=0):
        """totalflux_k's E > V(flux point) test for the wave (default on; off is
        the earlier form of the routine).  Before the first hphi/start."""
        self._check(self.L.mw3_set_flux_gate(self.h, wave, 1 if on else 0), "mw3_set_flux_gate")

    def set_ecoriolis(self, on, wave=0):
        """The electronic Coriolis Hamiltonian (mod_Hphi_eCoriolis_01y2.f) for the
        wave: channels of equal Omega whose Lambda differ by one couple through
        j^2.  Default off.  Before the first hphi/start."""
        self._check(self.L.mw3_set_ecoriolis(self.h, wave, 1 if on else 0), "mw3_set_ecoriolis")

    CHOICES = ("dst", "x_transposed", "angular", "angular_chunk")
    TUNE_SCOPES = {"layout": 1, "form": 2, "all": 3}

    def set_choices(self, choices):
        """Pin path choices (mw3_set_choices): a dict over CHOICES, missing keys
        keep the built-in rule.  Before start."""
        c = (ct.c_int32 * 4)(*[int(choices.get(k, 0 if k == "angular_chunk" else -1)) for k in self.CHOICES])
        self._check(self.L.mw3_set_choices(self.h, c), "mw3_set_choices")

    def choices(self):
        c = (ct.c_int32 * 4)()
        self._check(self.L.mw3_get_choices(self.h, c), "mw3_get_choices")
        return dict(zip(self.CHOICES, [int(v) for v in c]))

    def autotune(self, iterations=64, scope="layout"):
        """Time every distinct path the scope allows ("layout": bit-identical
        choices; "form": DST factorisation and angular form; "all") over
        `iterations` synthetic propagation iterations and keep the fastest.
        Before start; returns (choices, ms per iteration)."""
        c = (ct.c_int32 * 4)()
        ms = ct.c_double()
        self._check(self.L.mw3_autotune(self.h, int(iterations), self.TUNE_SCOPES[scope], c, ct.byref(ms)),
                    "mw3_autotune")
        return dict(zip(self.CHOICES, [int(v) for v in c])), ms.value

    def cvj_history(self, capacity):
        """Record Cvj (and Cvjprod) of every iteration in a device ring of
        ``capacity`` iterations (0: off)."""
        self._check(self.L.mw3_cvj_history(self.h, int(capacity)), "mw3_cvj_history")

    def download_cvj_history(self, n, wave=0):
        """(iterations [n], cvj [n][ncan][nj][nv], cvjprod [n][nom][njp][nvp] or
        None) of the last n recorded iterations, oldest first."""
        r = self.runs[wave]
        i = r.inp
        cvj = np.empty((n, r.ncan, i.jmax - i.jini + 1, i.nvmax - i.nvini + 1))
        shp = getattr(self, "_prodshape", {}).get(wave)
        cp = np.empty((n,) + shp) if shp is not None else None
        last = ct.c_int64()
        self._check(self.L.mw3_download_cvj_history(self.h, wave, n, _p(cvj), None if cp is None else _p(cp),
                                                     ct.byref(last)), "mw3_download_cvj_history")
        return np.arange(last.value - n + 1, last.value + 1), cvj, cp

    def psi_e(self, wave=0):
        """funE's zfe [nofe][ntot] complex: the energy-resolved wave functions
        accumulated over the iterations (SRC/mod_PsiE_01y2.f:92-123)."""
        r = self.runs[wave]
        efe = getattr(r, "efe_zot", None)
        nofe = 0 if efe is None else len(efe)
        if nofe == 0:
            raise Mw3Error("the wave has no funE energies (nofe = 0)")
        z = np.empty((nofe, self.ntot[wave], 2))
        self._check(self.L.mw3_download_accumulators(self.h, wave, None, None, None, None, _p(z)),
                    "mw3_download_accumulators")
        return z[..., 0] + 1j * z[..., 1]

    def tables(self, wave=0):
        r = self.runs[wave]
        i = r.inp
        nj, nv = i.jmax - i.jini + 1, i.nvmax - i.nvini + 1
        nopr1 = np.empty(i.nangu, np.int32)
        etot, reac = np.empty(i.netot), np.empty(i.netot)
        s2f = np.empty((r.nelec, nj, nv, i.netot))
        a1, a2 = np.empty(i.npun1), np.empty(i.npun2)
        self._check(self.L.mw3_tables(self.h, wave, _p(nopr1, ct.c_int32), _p(etot), _p(reac), _p(s2f), _p(a1),
                                      _p(a2)), "mw3_tables")
        apaq = np.empty(i.netot)
        self._check(self.L.mw3_packet_energy_norm(self.h, wave, _p(apaq)), "mw3_packet_energy_norm")
        return dict(nopr1=nopr1, etot=etot, reacfct=reac, s2factor=s2f, absfr1=a1, absfr2=a2, apaqini=apaq)

    def kernel_launches(self):
        n = ct.c_int64()
        self._check(self.L.mw3_kernel_launches(self.h, ct.byref(n)), "mw3_kernel_launches")
        return n.value

    def path(self):
        """Kernels in use (after start): tensor-core radial DSTs, fused into one
        kernel per slab or not (as split-FP16 or 3xTF32 products), and the
        tensor-core angular contraction."""
        f = ct.c_int32()
        self._check(self.L.mw3_path_flags(self.h, ct.byref(f)), "mw3_path_flags")
        return {"tc_dst": bool(f.value & 1), "tc_dst_fused": bool(f.value & 4), "tc_angular": bool(f.value & 2),
                "dst_f16": bool(f.value & 8), "x_transposed": bool(f.value & 16), "rader": bool(f.value & 32)}

    def stream(self):
        """cudaStream_t of the context, as an integer handle."""
        s = ct.c_void_p()
        self._check(self.L.mw3_get_stream(self.h, ct.byref(s)), "mw3_get_stream")
        return s.value or 0

    def profile(self, enable=True):
        self._check(self.L.mw3_profile(self.h, 1 if enable else 0), "mw3_profile")

    def stage_times(self):
        """Accumulated per-stage milliseconds since profiling was enabled."""
        ms = np.zeros(len(STAGES))
        n = ct.c_int64()
        self._check(self.L.mw3_stage_times(self.h, _p(ms), ct.byref(n)), "mw3_stage_times")
        return dict(zip(STAGES, ms)), n.value

    def close(self):
        if getattr(self, "h", None):
            self.L.mw3_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
