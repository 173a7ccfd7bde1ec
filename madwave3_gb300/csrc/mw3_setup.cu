// Host-side construction of the per-wave tables the replaced Fortran modules
// build once at start-up:
//   Tradial             SRC/mod_Hphi_01y2.f:487-620   (DST lengths, momenta)
//   angkinj2            SRC/mod_Hphi_01y2.f:166-311   (j^2 scalars per (r1, j))
//   bfgridl2mat         SRC/mod_Hphi_01y2.f:315-484   (l^2 Omega-coupling scalars per (R, j))
//   ini_absorcion       SRC/mod_absorcion_01y2.f:28-107
//   ini_flux            SRC/mod_flux_01y2.f:54-334
//   Smatini_col         SRC/mod_flux_01y2.f:392-524
// The angular matrices themselves are assembled on the device from these
// scalars and Djmmp (mw3_kernels.cu).
#include <math.h>
#include <string.h>

#include <algorithm>

#include "mw3_internal.h"

namespace mw3 {

static const double kPi = 3.14159265358979323846;   // dacos(-1.d0)

// integer power by binary powering (the order gfortran's powi uses)
static double powi(double x, int n)
{
    unsigned m = n < 0 ? -n : n;
    double y = (m % 2) ? x : 1.0;
    while (m >>= 1) {
        x = x * x;
        if (m % 2) y = y * x;
    }
    return n < 0 ? 1.0 / y : y;
}

// Smallest 2^a 3^b 5^c 7^d 11^e that is >= nin and within ntot of it, capped at
// ntot (noptFFT, liboctdyn.f:1033-1117).  Products wrap at 32 bits like the
// reference's default integers.
int noptfft(int nin, int ntot)
{
    const int base[5] = {2, 3, 5, 7, 11};
    int nexp[5];
    for (int q = 0; q < 5; q++) {
        int v = 1, e = 0;
        for (e = 0; e <= 100; e++) {
            v *= base[q];
            if (v > ntot) break;
        }
        nexp[q] = e;
    }
    int nout = 1, imin = ntot;
    int pw[5];
    for (int e11 = 0; e11 <= nexp[4]; e11++)
        for (int e7 = 0; e7 <= nexp[3]; e7++)
            for (int e5 = 0; e5 <= nexp[2]; e5++)
                for (int e3 = 0; e3 <= nexp[1]; e3++)
                    for (int e2 = 0; e2 <= nexp[0]; e2++) {
                        int ex[5] = {e2, e3, e5, e7, e11};
                        for (int q = 0; q < 5; q++) {
                            pw[q] = 1;
                            for (int t = 0; t < ex[q]; t++) pw[q] *= base[q];
                        }
                        uint32_t u = (uint32_t)pw[0] * (uint32_t)pw[1];
                        u *= (uint32_t)pw[2];
                        u *= (uint32_t)pw[3];
                        u *= (uint32_t)pw[4];
                        int i = (int)(int32_t)u;
                        int idis = i - nin;
                        if (idis >= 0 && idis < imin) {
                            nout = i;
                            imin = idis;
                        }
                    }
    if (nout > ntot) nout = ntot;
    return nout;
}

// p^2/(2 mu) of the sine basis with n points spaced like box/(n-1)
// (sinmom, liboctdyn.f:1004-1031)
static void sinmom_p2(double box, int npun, double xmred, double hbr, double *p2r)
{
    double dpi = 2.0 * kPi;
    double hbrxm = 0.5 * hbr * hbr / xmred;
    double ah = box / (double)(npun - 1);
    double b2 = 2.0 * ((double)npun + 1.0) * ah;
    for (int ir = 1; ir <= npun; ir++) {
        double p = dpi * (double)ir / b2;
        p2r[ir - 1] = p * p * hbrxm;
    }
}

// momenta of the FFT grid (fftmom, liboctdyn.f:1119-1152)
static void fftmom_p(double box, int npun, double *pr)
{
    double dpi = 2.0 * kPi;
    double ah = box / (double)(npun - 1);
    double b2 = ah * (double)npun;
    for (int ir = 1; ir <= npun; ir++) {
        int iii = (ir <= npun / 2) ? ir - 1 : ir - npun - 1;
        pr[ir - 1] = dpi * (double)iii / b2;
    }
}

// Ascending eigenvalues of a small symmetric matrix (cyclic Jacobi rotations).
static void sym_eigvals(int n, std::vector<double> a, double *ev)
{
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0.0;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) off += fabs(a[p * n + q]);
        if (off == 0.0) break;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) {
                double apq = a[p * n + q];
                if (apq == 0.0) continue;
                double theta = 0.5 * (a[q * n + q] - a[p * n + p]) / apq;
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
                for (int k = 0; k < n; k++) {
                    double akp = a[k * n + p], akq = a[k * n + q];
                    a[k * n + p] = cs * akp - sn * akq;
                    a[k * n + q] = sn * akp + cs * akq;
                }
                for (int k = 0; k < n; k++) {
                    double apk = a[p * n + k], aqk = a[q * n + k];
                    a[p * n + k] = cs * apk - sn * aqk;
                    a[q * n + k] = sn * apk + cs * aqk;
                }
            }
    }
    for (int i = 0; i < n; i++) ev[i] = a[i * n + i];
    std::sort(ev, ev + n);
}

// Riccati-Bessel functions F_l = x j_l(x), G_l = x y_l(x) (G ~ -cos(x - l pi/2)):
// the open-channel solutions BESPH2 returns (liboctdyn.f:743-835).  G by upward
// recurrence, F upward above x = l and by Miller's downward recurrence below.
void riccati_fg(int l, double x, double *f, double *g)
{
    double s = sin(x), c = cos(x);
    double g0 = -c, g1 = -c / x - s;
    if (l == 0) {
        *g = g0;
        *f = s;
        return;
    }
    double gm = g0, gc = g1;
    for (int k = 1; k < l; k++) {
        double gn = (2.0 * k + 1.0) / x * gc - gm;
        gm = gc;
        gc = gn;
    }
    *g = gc;
    if (x > (double)l) {
        double fm = s, fc = s / x - c;
        for (int k = 1; k < l; k++) {
            double fn = (2.0 * k + 1.0) / x * fc - fm;
            fm = fc;
            fc = fn;
        }
        *f = fc;
        return;
    }
    int nstart = l + 40 + (int)x;
    double fp = 0.0, fc = 1e-300, fl = 0.0;
    for (int k = nstart; k >= 1; k--) {
        double fn = (2.0 * k + 1.0) / x * fc - fp;
        fp = fc;
        fc = fn;
        if (k - 1 == l) fl = fc;
        if (fabs(fc) > 1e250) {
            fc *= 1e-250;
            fp *= 1e-250;
            fl *= 1e-250;
        }
    }
    double scale = (fabs(s) > fabs(s / x - c)) ? s / fc : (s / x - c) / fp;
    *f = fl * scale;
}

static inline double djv(const WaveTables &t, int na, int ne, int iom, int ielec, int j, int iang)
{
    return t.djmmp[(((size_t)iom * ne + (ielec - 1)) * (t.nangu2 + 1) + j) * na + (iang - 1)];
}

int build_wave_tables(Ctx &c, const mw3_wave &w, WaveTables &t, std::string &err)
{
    const mw3_grid &gr = c.grid;
    int n1 = c.n1, n2 = c.n2, na = c.na, ne = c.ne;
    double ah1 = (gr.rfin1 - gr.rmis1) / (double)(n1 - 1);
    double ah2 = (gr.rfin2 - gr.rmis2) / (double)(n2 - 1);
    // ---- copy scalars and arrays ----
    t.Jtot = w.Jtot; t.iparity = w.iparity; t.inc = w.inc; t.j0 = w.j0;
    t.iommin = w.iommin; t.iommax = w.iommax; t.ncan = w.ncan; t.nangu2 = w.nangu2;
    t.proj_j2_up = w.proj_j2_up;
    t.absr1 = w.absr1; t.absalp1 = w.absalp1; t.absr2 = w.absr2; t.absalp2 = w.absalp2;
    t.n1expo = w.n1expo; t.ninterv1 = w.ninterv1; t.n2expo = w.n2expo; t.ninterv2 = w.ninterv2;
    t.r1flux_ang = w.r1flux_ang; t.ekinmin = w.ekinmin; t.ekinmax = w.ekinmax;
    t.netot = w.netot; t.kminelastic = w.kminelastic; t.iphoto = w.iphoto; t.iprod = w.iprod;
    t.nvini = w.nvini; t.nvmax = w.nvmax; t.jini = w.jini; t.jmax = w.jmax;
    t.nvref = w.nvref; t.jref = w.jref; t.iomref = w.iomref; t.ielecref = w.ielecref;
    t.xm1reac = w.xm1reac; t.xm2reac = w.xm2reac; t.rcolini = w.rcolini; t.alpha0 = w.alpha0;
    t.xk0 = w.xk0; t.factor0 = w.factor0; t.xmasa0 = w.xmasa0; t.il0 = w.il0; t.nofe = w.nofe;
    if (w.proj_j2_up != 0) {
        err = "Proj_j2_up != 0 reads Wigner values the reference never sets; not supported";
        return MW3_ERR_UNSUPPORTED;
    }
    if (w.iphoto < 0 || w.iphoto > 2) {
        err = "iphoto must be 0 (collision), 1 (dipole transition) or 2 (bright approximation)";
        return MW3_ERR_UNSUPPORTED;
    }
    if (w.iprod == 1) {
        err = "product-Jacobi propagation (iprod=1) is not supported";
        return MW3_ERR_UNSUPPORTED;
    }
    if (w.ncan <= 0 || w.inc < 1 || w.inc > 2 || w.nangu2 != na * w.inc || w.netot < 2) {
        err = "inconsistent wave sizes";
        return MW3_ERR_ARG;
    }
    if (w.jmax < w.jini || w.nvmax < w.nvini || w.jmax > w.nangu2) {
        err = "inconsistent j/v ranges";
        return MW3_ERR_ARG;
    }
    int nc = w.ncan;
    t.iombas.assign(w.iombas, w.iombas + nc);
    t.nelebas.assign(w.nelebas, w.nelebas + nc);
    t.nojbas.assign(w.nojbas, w.nojbas + nc);
    t.j00.assign(w.j00, w.j00 + nc);
    t.jbas.assign(w.jbas, w.jbas + (size_t)nc * na);
    t.iomdiat.assign(w.iomdiat, w.iomdiat + ne);
    t.iomatom.assign(w.iomatom, w.iomatom + ne);
    t.sigdiat.assign(w.sigdiat, w.sigdiat + ne);
    t.sigatom.assign(w.sigatom, w.sigatom + ne);
    t.djmmp.assign(w.djmmp, w.djmmp + (size_t)(w.Jtot + 1) * ne * (w.nangu2 + 1) * na);
    t.nj = w.jmax - w.jini + 1;
    t.nv = w.nvmax - w.nvini + 1;
    t.nobc.assign(w.nobc, w.nobc + (size_t)ne * t.nj);
    t.ediat.assign(w.ediat, w.ediat + (size_t)ne * t.nj * t.nv);
    t.fd.assign(w.fd, w.fd + (size_t)ne * t.nj * t.nv * n1);
    if (w.nofe > 0) t.efe.assign(w.efe, w.efe + w.nofe);
    for (int b = 0; b < nc; b++) {
        if (t.nelebas[b] < 1 || t.nelebas[b] > ne || t.iombas[b] < 0 || t.iombas[b] > w.Jtot ||
            t.iombas[b] < w.iommin || t.iombas[b] > w.iommax || t.nojbas[b] < 1 || t.nojbas[b] > na) {
            err = "bad block description";
            return MW3_ERR_ARG;
        }
        for (int k = 0; k < t.nojbas[b]; k++)
            if (t.jbas[(size_t)b * na + k] < 0 || t.jbas[(size_t)b * na + k] > w.nangu2) {
                err = "jbas out of range";
                return MW3_ERR_ARG;
            }
    }

    // ---- flat layout (indtotproc, one process) ----
    t.offs.assign((size_t)na * nc, 0);
    int64_t cnt = 0;
    for (int ia = 0; ia < na; ia++) {
        int iang = na - ia;
        for (int b = 0; b < nc; b++) {
            t.offs[(size_t)(iang - 1) * nc + b] = cnt;
            cnt += c.npunreal[iang - 1];
        }
    }
    t.ntot = cnt;

    // ---- Tradial ----
    t.nopr1.assign(na, 1);
    t.p2r1.assign((size_t)na * n1, 0.0);
    t.p2r2.assign((size_t)na * n2, 0.0);
    for (int a = 0; a < na; a++) {
        int np = c.npunreal[a];
        int mn = n1, mx = 0;
        for (int ir = 0; ir < np; ir++) {
            int ir1 = c.indr1[(size_t)a * c.npt + ir];
            mn = std::min(mn, ir1);
            mx = std::max(mx, ir1);
        }
        t.nopr1[a] = mx - mn + 1;
    }
    for (int e = 0; e < ne; e++)
        for (int a = 0; a < na; a++) {
            int nn = noptfft(t.nopr1[a], n1);
            if (nn < gr.npun1min) nn = gr.npun1min;
            t.nopr1[a] = nn;
            if (n1 > 1) sinmom_p2((double)(nn - 1) * ah1, nn, gr.xm1red, gr.hbr, &t.p2r1[(size_t)a * n1]);
            sinmom_p2((double)(n2 - 1) * ah2, n2, gr.xm2red, gr.hbr, &t.p2r2[(size_t)a * n2]);
        }
    for (int a = 0; a < na; a++)
        if (t.nopr1[a] > n1 || t.nopr1[a] < 1) {
            err = "DST length in r1 exceeds npun1 (npun1min too large?)";
            return MW3_ERR_UNSUPPORTED;
        }

    // ---- angkinj2 scalars: yyy(ir1, k) = min((j(j+1)-Omd^2) hbar^2/2 / (mu r1^2), rotcut) ----
    t.yj2.assign((size_t)nc * n1 * na, 0.0);
    int jjjmax = (na - 1) * w.inc;
    if (na > 1)
        for (int b = 0; b < nc; b++) {
            int iomdi = t.iomdiat[t.nelebas[b] - 1];
            for (int ir1 = 1; ir1 <= n1; ir1++) {
                double r1 = gr.rmis1 + (double)(ir1 - 1) * ah1;
                for (int k = 0; k < t.nojbas[b]; k++) {
                    int jb = t.jbas[(size_t)b * na + k];
                    if (jb > jjjmax) continue;
                    double xj = (double)jb, xom = (double)iomdi;
                    double xkinj = (xj * (xj + 1.0) - xom * xom) * gr.hbr * gr.hbr * 0.5;
                    double yyy = xkinj / (gr.xm1red * r1 * r1);
                    if (yyy > gr.rotcutmax) yyy = gr.rotcutmax;
                    t.yj2[((size_t)b * n1 + (ir1 - 1)) * na + k] = yyy;
                }
            }
        }

    // ---- bfgridl2mat scalars ----
    t.nom = w.iommax - w.iommin + 1;
    t.nj2 = (na - 1) / 1 + 1;                    // j index 0..na-1 -> j = j0 + jidx*inc
    int nom = t.nom;
    t.l2tab.assign((size_t)ne * t.nj2 * n2 * nom * nom, 0.0);
    t.l2used.assign((size_t)ne * t.nj2 * nom * nom, 0);
    double facmass = gr.hbr * gr.hbr * 0.5 / gr.xm2red;
    for (int ielec = 1; ielec <= ne; ielec++) {
        int sigelec = 1;
        if (t.sigdiat[ielec - 1] == -1.0 || t.sigatom[ielec - 1] == -1.0) sigelec = -1;
        for (int jidx = 0;; jidx++) {
            int j = w.j0 + jidx * w.inc;
            if (j > (na - 1) * w.inc) break;
            int iom0 = w.iommin;
            int pj = (w.Jtot % 2) ? -1 : 1;
            if (w.iparity != sigelec * pj && w.iommin == 0) iom0 = 1;
            if (iom0 > j) continue;
            int iom1 = std::min(j, w.iommax);
            int nnn = iom1 - iom0 + 1;
            if (nnn <= 0) continue;
            // l2mat (liboctdyn.f:1944-1990)
            std::vector<double> bfl((size_t)nnn * nnn, 0.0);
            double xj = (double)j;
            for (int iom = iom0; iom <= iom1; iom++)
                for (int jom = iom0; jom <= iom1; jom++) {
                    double xk = 0.0;
                    if (iom == jom) {
                        double x1 = xj * (xj + 1.0);
                        double x2 = (double)(w.Jtot * (w.Jtot + 1) - 2 * iom * jom);
                        xk = (x1 + x2) * facmass;
                    } else if (abs(iom - jom) == 1) {
                        double x1 = (double)(w.Jtot * (w.Jtot + 1) - iom * jom);
                        double x2 = xj * (xj + 1.0) - (double)(iom * jom);
                        double x12 = sqrt(x1 * x2);
                        xk = -x12 * facmass;
                        if (iom * jom == 0) xk = xk * sqrt(2.0);
                    }
                    bfl[(size_t)(iom - iom0) * nnn + (jom - iom0)] = xk;
                }
            double yylmin, yylmax, yylmean;
            if (nnn > 1) {
                std::vector<double> ev(nnn);
                sym_eigvals(nnn, bfl, ev.data());
                yylmin = ev[0];
                yylmax = ev[nnn - 1];
                yylmean = 0.5 * (yylmin + yylmax);
            } else {
                yylmin = bfl[0];
                yylmax = yylmin;
                yylmean = yylmin;
            }
            (void)yylmax;
            for (int iom = iom0; iom <= iom1; iom++)
                for (int jom = iom0; jom <= iom1; jom++)
                    if (abs(iom - jom) <= 1)
                        t.l2used[(((size_t)(ielec - 1) * t.nj2 + jidx) * nom + (iom - w.iommin)) * nom + (jom - w.iommin)] = 1;
            for (int ir2 = 1; ir2 <= n2; ir2++) {
                double r2 = gr.rmis2 + (double)(ir2 - 1) * ah2;
                double r2eff = r2;
                double emeaneff = yylmean / (r2 * r2);
                if (emeaneff > gr.rotcutmax) r2eff = sqrt(fabs(yylmean / gr.rotcutmax));
                for (int iom = iom0; iom <= iom1; iom++)
                    for (int jom = iom0; jom <= iom1; jom++) {
                        double bv = bfl[(size_t)(iom - iom0) * nnn + (jom - iom0)];
                        double v = 0.0;
                        if (fabs(bv) > 1e-8 && r2eff > 1e-3) v = bv / (r2eff * r2eff);
                        t.l2tab[((((size_t)(ielec - 1) * t.nj2 + jidx) * n2 + (ir2 - 1)) * nom + (iom - w.iommin)) * nom +
                                (jom - w.iommin)] = v;
                    }
            }
        }
    }

    // ---- ini_absorcion ----
    t.absfr1.assign(n1, 1.0);
    t.absfr2.assign(n2, 1.0);
    t.ir1abs = n1;
    t.ir2abs = n2;
    for (int ir1 = 1; ir1 <= n1; ir1++) {
        double r1 = (double)(ir1 - 1) * ah1 + gr.rmis1;
        double f1 = 1.0;
        if (r1 >= w.absr1) {
            if (ir1 < t.ir1abs) t.ir1abs = ir1;
            double delta = (r1 - w.absr1) / (double)w.ninterv1;
            f1 = exp(-(w.absalp1 * powi(delta, w.n1expo)));
        }
        t.absfr1[ir1 - 1] = f1;
    }
    for (int ir2 = 1; ir2 <= n2; ir2++) {
        double r2 = (double)(ir2 - 1) * ah2 + gr.rmis2;
        double f2 = 1.0;
        if (r2 >= w.absr2) {
            if (ir2 < t.ir2abs) t.ir2abs = ir2;
            double delta = (r2 - w.absr2) / (double)w.ninterv2;
            f2 = exp(-(w.absalp2 * powi(delta, w.n2expo)));
        }
        t.absfr2[ir2 - 1] = f2;
    }

    // ---- ini_flux: derivative row, flux line per angle, flux points ----
    t.nflux = 0;
    t.ir1flux.assign(na, 0);
    t.zar1flux.assign((size_t)2 * n1, 0.0);
    if (n1 > 1) {
        double r1flux = w.r1flux_ang;
        t.ir4flux = 0;
        for (int ir1 = 1; ir1 <= n1; ir1++) {
            double r1 = gr.rmis1 + (double)(ir1 - 1) * ah1;
            if (r1 <= r1flux && ir1 > t.ir4flux) t.ir4flux = ir1;
        }
        std::vector<double> xpr1(n1);
        fftmom_p((double)(n1 - 1) * ah1, n1, xpr1.data());
        for (int m = 1; m <= n1; m++) {
            double d2r = (double)(t.ir4flux - m) * ah1;
            double zr = 0.0, zi = 0.0;
            for (int k = 1; k <= n1; k++) {
                double xk = xpr1[k - 1];
                double cs = cos(xk * d2r), sn = sin(xk * d2r);
                // (0 + i xk)(cs + i sn)
                zr = zr + (0.0 * cs - xk * sn);
                zi = zi + (0.0 * sn + xk * cs);
            }
            t.zar1flux[2 * (m - 1)] = zr / (double)(2 * n1);
            t.zar1flux[2 * (m - 1) + 1] = zi / (double)(2 * n1);
        }
        for (int a = 0; a < na; a++) {
            int np = c.npunreal[a];
            for (int ir = 0; ir < np; ir++) {
                int ir1 = c.indr1[(size_t)a * c.npt + ir];
                double r1 = (double)(ir1 - 1) * ah1 + gr.rmis1;
                if (r1 <= r1flux && ir1 > t.ir1flux[a]) t.ir1flux[a] = ir1;
            }
        }
        // flux points in the reference's order: angle (flat order), block, point
        std::vector<int> rowmap((size_t)n2);
        for (int ia = 0; ia < na; ia++) {
            int a = na - 1 - ia;
            int np = c.npunreal[a];
            for (int b = 0; b < nc; b++) {
                int ielec = t.nelebas[b];
                for (int ir = 0; ir < np; ir++) {
                    int ir1 = c.indr1[(size_t)a * c.npt + ir];
                    if (ir1 != t.ir1flux[a]) continue;
                    int ir2 = c.indr2[(size_t)a * c.npt + ir];
                    t.fl_idx.push_back(t.offs[(size_t)a * nc + b] + ir);
                    t.fl_block.push_back(b);
                    t.potiflux.push_back(
                        c.vvv[(((size_t)(ielec - 1) * ne + (ielec - 1)) * na + a) * c.npt + ir]);
                    // derivative terms: every stored point of (block, angle, ir2)
                    t.fl_dptr.push_back((int)t.fl_didx.size());
                    for (int jr = 0; jr < np; jr++)
                        if (c.indr2[(size_t)a * c.npt + jr] == ir2) {
                            t.fl_didx.push_back(t.offs[(size_t)a * nc + b] + jr);
                            t.fl_dir1.push_back(c.indr1[(size_t)a * c.npt + jr] - 1);
                        }
                }
            }
        }
        t.fl_dptr.push_back((int)t.fl_didx.size());
        t.nflux = (int)t.fl_idx.size();
    }

    // ---- Smatini: reference channel; Smatini_col ----
    t.icanref = -1;
    for (int b = 0; b < nc; b++)
        if (t.nelebas[b] == w.ielecref && t.iombas[b] == abs(w.iomref)) t.icanref = b;
    if (t.icanref < 0) {
        err = "icanref can not be set (no block for ielecref, |iomref|)";
        return MW3_ERR_ARG;
    }
    int netot = w.netot;
    double estep = (w.ekinmax - w.ekinmin) / (double)(netot - 1);
    if (w.iphoto >= 1) {
        // Smatini_photo (SRC/mod_flux_01y2.f:526-581): no collision packet to divide
        // by; the normalisation of the initial packet (photonorm) is the host's
        t.etot.assign(netot, 0.0);
        t.reacfct.assign(netot, 0.25 / kPi / w.xm1reac);
        t.apaqini.assign(netot, 0.0);
        t.s2factor.assign((size_t)ne * t.nj * t.nv * netot, 0.0);
        for (int ie = 0; ie < netot; ie++) {
            t.etot[ie] = w.ekinmin + (double)ie * estep;
            for (int e = 0; e < ne; e++)
                for (int jj = 0; jj < t.nj; jj++)
                    for (int iv = 0; iv < t.nv; iv++) {
                        double ekf = t.etot[ie] - t.ediat[((size_t)e * t.nj + jj) * t.nv + iv];
                        double pfin = ekf > 0.0 ? sqrt(ekf * w.xm2reac * 2.0 / gr.hbr / gr.hbr) : 0.0;
                        t.s2factor[(((size_t)e * t.nj + jj) * t.nv + iv) * netot + ie] = 4.0 * pfin / (kPi * w.xm2reac);
                    }
        }
    } else {
    const int npunt = 1000;
    std::vector<double> rg(npunt);
    double ahgauss = (gr.rfin2 - gr.rmis2) / (double)(npunt - 1);
    for (int ir2 = 1; ir2 <= npunt; ir2++) {
        double r2 = gr.rmis2 + (double)(ir2 - 1) * ahgauss;
        double gg = cos((r2 - w.rcolini) * w.xk0) * sqrt(2.0);
        double xr2 = gg * w.factor0 * exp(-(r2 - w.rcolini) * (r2 - w.rcolini) / w.alpha0 / w.alpha0);
        rg[ir2 - 1] = xr2 / sqrt(2.0);
    }
    double pepe = (double)(w.il0 * (w.il0 + 1));
    double rr = w.rcolini + 1.0;
    double erot = gr.hbr * gr.hbr * pepe * 0.5 / (rr * rr * w.xmasa0);
    t.etot.assign(netot, 0.0);
    t.reacfct.assign(netot, 0.0);
    t.apaqini.assign(netot, 0.0);
    t.s2factor.assign((size_t)ne * t.nj * t.nv * netot, 0.0);
    for (int ie = 0; ie < netot; ie++) {
        t.etot[ie] = w.ekinmin + (double)ie * estep;
        double ek = t.etot[ie];
        double paqini = 0.0, pini = 0.0;
        if (ek > 0.0 && ek > erot) {
            pini = sqrt(ek * w.xmasa0 * 2.0 / gr.hbr / gr.hbr);
            double zr = 0.0, zi = 0.0;
            for (int ir2 = 1; ir2 <= npunt; ir2++) {
                double rx = gr.rmis2 + (double)(ir2 - 1) * ahgauss;
                double fb, gb;
                riccati_fg(w.il0, rx * pini, &fb, &gb);
                if (fabs(fb) > 1e-20) {
                    zr += rg[ir2 - 1] * (-gb);
                    zi += rg[ir2 - 1] * fb;
                }
            }
            zr = zr * ahgauss / 2.0 / kPi;
            zi = zi * ahgauss / 2.0 / kPi;
            paqini = zr * zr + zi * zi;
        }
        t.apaqini[ie] = paqini;
        for (int e = 0; e < ne; e++)
            for (int jj = 0; jj < t.nj; jj++)
                for (int iv = 0; iv < t.nv; iv++) {
                    double ekf = t.etot[ie] - t.ediat[((size_t)e * t.nj + jj) * t.nv + iv];
                    double pfin = ekf > 0.0 ? sqrt(ekf * w.xm2reac * 2.0 / gr.hbr / gr.hbr) : 0.0;
                    t.s2factor[(((size_t)e * t.nj + jj) * t.nv + iv) * netot + ie] =
                        (paqini < 1e-10) ? 0.0 : gr.hbr * gr.hbr * pfin * pini / (2.0 * paqini) / w.xm2reac / w.xmasa0;
                }
        t.reacfct[ie] =
            (paqini < 1e-10) ? 0.0 : gr.hbr * gr.hbr * pini / paqini / w.xmasa0 / w.xm1reac / 4.0 / kPi / kPi;
    }
    }   // collision (Smatini_col)

    // ---- Cvjflux_k: point at (ir1, ir2abs) for every angle ----
    t.r2abs_map.assign((size_t)na * n1, -1);
    for (int a = 0; a < na; a++) {
        int np = c.npunreal[a];
        for (int ir = 0; ir < np; ir++)
            if (c.indr2[(size_t)a * c.npt + ir] == t.ir2abs)
                t.r2abs_map[(size_t)a * n1 + (c.indr1[(size_t)a * c.npt + ir] - 1)] = ir;
    }
    (void)djv;
    return MW3_OK;
}

// Channel pairs of the electronic Coriolis variant and their j-basis scalars
// (angkinj2 of mod_Hphi_eCoriolis_01y2.f:226-285): a source channel b couples to a
// target b2 of equal Omega and sigma whose diatomic Lambda differs by one, through
// the basis indices k at which both hold the same j:
//   y(r1, k) = min(sqrt(L^2 + L'^2) sqrt(j(j+1) - |L L'|) hbar^2 [x sqrt 2 if L or L' is 0]
//                  / (mu r1^2), rotcutmax),
// later transformed with the source's Djmmp on both sides.  Pairs are listed
// target-major; src/dst are wave-local channels, y is [pair][npun1][nangu].
void ecor_pairs(const Ctx &c, const WaveTables &t, std::vector<int> &src, std::vector<int> &dst,
                std::vector<double> &y)
{
    const mw3_grid &gr = c.grid;
    int n1 = c.n1, na = c.na, nc = t.ncan;
    double ah1 = (gr.rfin1 - gr.rmis1) / (double)(n1 - 1);
    int jjjmax = (na - 1) * t.inc;
    src.clear();
    dst.clear();
    y.clear();
    if (!t.ecor || na <= 1) return;
    for (int bd = 0; bd < nc; bd++) {
        int jelec = t.nelebas[bd], jomdi = t.iomdiat[jelec - 1];
        for (int b = 0; b < nc; b++) {
            int ielec = t.nelebas[b], iomdi = t.iomdiat[ielec - 1];
            if (b == bd || t.iombas[b] != t.iombas[bd]) continue;
            if (t.sigdiat[ielec - 1] != t.sigdiat[jelec - 1] || std::abs(jomdi - iomdi) != 1) continue;
            src.push_back(b);
            dst.push_back(bd);
            size_t p0 = y.size();
            y.resize(p0 + (size_t)n1 * na, 0.0);
            int nk = std::min(t.nojbas[b], t.nojbas[bd]);
            for (int ir1 = 1; ir1 <= n1; ir1++) {
                double r1 = gr.rmis1 + (double)(ir1 - 1) * ah1;
                for (int k = 0; k < nk; k++) {
                    int jb = t.jbas[(size_t)b * na + k];
                    if (jb != t.jbas[(size_t)bd * na + k] || jb > jjjmax) continue;
                    double xj = (double)jb;
                    double xlam = sqrt((double)(iomdi * iomdi) + (double)(jomdi * jomdi));
                    double xom = sqrt(xj * (xj + 1) - (double)std::abs(jomdi * iomdi));
                    double xkinj = xlam * xom * gr.hbr * gr.hbr;
                    if (jomdi == 0 || iomdi == 0) xkinj = xkinj * sqrt(2.0);
                    double yyy = xkinj / (gr.xm1red * r1 * r1);
                    if (yyy > gr.rotcutmax) yyy = gr.rotcutmax;
                    y[p0 + (size_t)(ir1 - 1) * na + k] = yyy;
                }
            }
        }
    }
}

}  // namespace mw3
