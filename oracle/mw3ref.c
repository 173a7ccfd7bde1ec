/*
 * mw3ref.c -- CPU oracle for the madwave3 Chebyshev hot path.
 * TEST INFRASTRUCTURE ONLY (checker and timed CPU baseline); see mw3ref.h for
 * the list of restated reference routines.  Every loop below follows the
 * cited Fortran loop nest, including its operation order where that fixes the
 * rounding, and its quirks (points with ir1 > nopr1 that the DST leaves out,
 * the k = 0/1 terms the main program never accumulates).
 */
#include "mw3ref.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* pi = dacos(-1.d0) in the reference; this literal is that double */
#define MW3_PI 3.14159265358979323846

typedef struct { double re, im; } cplx;

static inline cplx cmul(cplx a, cplx b) { cplx r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; return r; }
static inline cplx cadd(cplx a, cplx b) { cplx r = {a.re + b.re, a.im + b.im}; return r; }

/* ---------------------------------------------------------------------- */
/* DST-I (FFTW RODFT00): y_k = 2 sum_j x_j sin(pi (j+1)(k+1)/(n+1))          */
/* ---------------------------------------------------------------------- */

typedef struct fftplan {
    int n;            /* DFT length */
    int m;            /* power-of-two length (n itself when n is a power of two) */
    int pow2;
    cplx *tw;         /* twiddles of the length-m radix-2 FFT */
    cplx *chirp;      /* Bluestein chirp w_k = exp(-i pi k^2 / n) */
    cplx *bhat;       /* FFT of the conjugate chirp filter */
    struct fftplan *next;
} fftplan;

static void fft_pow2(cplx *a, int m, const cplx *tw, int inverse)
{
    /* iterative radix-2 Cooley-Tukey, bit-reversed input permutation */
    for (int i = 1, j = 0; i < m; i++) {
        int bit = m >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) { cplx t = a[i]; a[i] = a[j]; a[j] = t; }
    }
    for (int len = 2; len <= m; len <<= 1) {
        int step = m / len;
        for (int i = 0; i < m; i += len) {
            for (int k = 0; k < len / 2; k++) {
                cplx w = tw[k * step];
                if (inverse) w.im = -w.im;
                cplx u = a[i + k], v = cmul(a[i + k + len / 2], w);
                a[i + k].re = u.re + v.re; a[i + k].im = u.im + v.im;
                a[i + k + len / 2].re = u.re - v.re; a[i + k + len / 2].im = u.im - v.im;
            }
        }
    }
}

static fftplan *plan_new(int n)
{
    fftplan *p = (fftplan *)calloc(1, sizeof(fftplan));
    p->n = n;
    int m = 1;
    while (m < n) m <<= 1;
    p->pow2 = (m == n);
    if (!p->pow2) { m = 1; while (m < 2 * n - 1) m <<= 1; }
    p->m = m;
    p->tw = (cplx *)malloc(sizeof(cplx) * m);
    for (int k = 0; k < m; k++) {
        double a = -2.0 * MW3_PI * (double)k / (double)m;
        p->tw[k].re = cos(a); p->tw[k].im = sin(a);
    }
    if (!p->pow2) {
        p->chirp = (cplx *)malloc(sizeof(cplx) * n);
        p->bhat = (cplx *)calloc(m, sizeof(cplx));
        for (int k = 0; k < n; k++) {
            long long kk = ((long long)k * k) % (2LL * n);
            double a = -MW3_PI * (double)kk / (double)n;
            p->chirp[k].re = cos(a); p->chirp[k].im = sin(a);
        }
        for (int k = 0; k < n; k++) {
            cplx c = {p->chirp[k].re, -p->chirp[k].im};
            p->bhat[k] = c;
            if (k) p->bhat[m - k] = c;
        }
        fft_pow2(p->bhat, m, p->tw, 0);
    }
    return p;
}

static void plan_free(fftplan *p)
{
    while (p) {
        fftplan *q = p->next;
        free(p->tw); free(p->chirp); free(p->bhat); free(p);
        p = q;
    }
}

/* forward DFT of length p->n in place; work has room for p->m entries */
static void dft(fftplan *p, cplx *x, cplx *work)
{
    if (p->pow2) { fft_pow2(x, p->n, p->tw, 0); return; }
    int n = p->n, m = p->m;
    for (int k = 0; k < n; k++) work[k] = cmul(x[k], p->chirp[k]);
    for (int k = n; k < m; k++) { work[k].re = 0; work[k].im = 0; }
    fft_pow2(work, m, p->tw, 0);
    for (int k = 0; k < m; k++) work[k] = cmul(work[k], p->bhat[k]);
    fft_pow2(work, m, p->tw, 1);
    double s = 1.0 / (double)m;
    for (int k = 0; k < n; k++) {
        cplx v = {work[k].re * s, work[k].im * s};
        x[k] = cmul(v, p->chirp[k]);
    }
}

typedef struct {
    fftplan *plans;
} dstcache;

static fftplan *get_plan(dstcache *c, int n)
{
    for (fftplan *p = c->plans; p; p = p->next) if (p->n == n) return p;
    fftplan *p = plan_new(n);
    p->next = c->plans;
    c->plans = p;
    return p;
}

/* Two DST-Is of length n at once through one complex DFT of the odd extensions
   (length 2(n+1)): for odd real a, b, DFT(a + i b)_k = 2 Sb_k - 2 i Sa_k. */
static void dst1_pair_fft(dstcache *c, int n, const double *xa, const double *xb,
                          double *ya, double *yb, cplx *buf, cplx *work)
{
    int N = 2 * (n + 1);
    fftplan *p = get_plan(c, N);
    buf[0].re = 0; buf[0].im = 0;
    buf[n + 1].re = 0; buf[n + 1].im = 0;
    for (int j = 0; j < n; j++) {
        double a = xa[j], b = xb ? xb[j] : 0.0;
        buf[j + 1].re = a; buf[j + 1].im = b;
        buf[N - 1 - j].re = -a; buf[N - 1 - j].im = -b;
    }
    dft(p, buf, work);
    for (int k = 0; k < n; k++) {
        ya[k] = -buf[k + 1].im;
        if (yb) yb[k] = buf[k + 1].re;
    }
}

static void dst1_direct(int n, const double *x, double *y)
{
    for (int k = 0; k < n; k++) {
        double s = 0.0;
        for (int j = 0; j < n; j++) {
            long long m = ((long long)(j + 1) * (k + 1)) % (2LL * (n + 1));
            s += x[j] * sin(MW3_PI * (double)m / (double)(n + 1));
        }
        y[k] = 2.0 * s;
    }
}

void mw3ref_dst1(int n, const double *x, double *y, int mode)
{
    if (mode == 1) { dst1_direct(n, x, y); return; }
    dstcache c = {0};
    int N = 2 * (n + 1);
    int m = 1; while (m < 2 * N) m <<= 1;
    cplx *buf = (cplx *)malloc(sizeof(cplx) * N), *work = (cplx *)malloc(sizeof(cplx) * m);
    dst1_pair_fft(&c, n, x, NULL, y, NULL, buf, work);
    free(buf); free(work);
    plan_free(c.plans);
}

/* ---------------------------------------------------------------------- */
/* small library pieces                                                   */
/* ---------------------------------------------------------------------- */

/* integer power by binary powering, the order libgcc's __powidf2 uses */
static double powi(double x, int n)
{
    unsigned m = (n < 0) ? -n : n;
    double y = (m % 2) ? x : 1.0;
    while (m >>= 1) { x = x * x; if (m % 2) y = y * x; }
    return (n < 0) ? 1.0 / y : y;
}

/* noptFFT (liboctdyn.f:1033-1117): smallest 2^a 3^b 5^c 7^d 11^e >= nin within
   ntot of it, capped at ntot; products wrap at 32 bits as the Fortran integers do */
static int noptfft(int nin, int ntot)
{
    int nexp[5], base[5] = {2, 3, 5, 7, 11};
    for (int q = 0; q < 5; q++) {
        int v = 1, e;
        for (e = 0; e <= 100; e++) { v *= base[q]; if (v > ntot) break; }
        nexp[q] = e;
    }
    int nout = 1, imin = ntot;
    for (int n11 = 0; n11 <= nexp[4]; n11++) {
        int i11 = 1; for (int t = 0; t < n11; t++) i11 *= 11;
        for (int n7 = 0; n7 <= nexp[3]; n7++) {
            int i7 = 1; for (int t = 0; t < n7; t++) i7 *= 7;
            for (int n5 = 0; n5 <= nexp[2]; n5++) {
                int i5 = 1; for (int t = 0; t < n5; t++) i5 *= 5;
                for (int n3 = 0; n3 <= nexp[1]; n3++) {
                    int i3 = 1; for (int t = 0; t < n3; t++) i3 *= 3;
                    for (int n2 = 0; n2 <= nexp[0]; n2++) {
                        int i2 = 1; for (int t = 0; t < n2; t++) i2 *= 2;
                        uint32_t u = (uint32_t)i2 * (uint32_t)i3;
                        u = u * (uint32_t)i5; u = u * (uint32_t)i7; u = u * (uint32_t)i11;
                        int i = (int)(int32_t)u;
                        int idis = i - nin;
                        if (idis >= 0 && idis < imin) { nout = i; imin = idis; }
                    }
                }
            }
        }
    }
    if (nout > ntot) nout = ntot;
    return nout;
}

/* sinmom (liboctdyn.f:1004-1031); box is recomputed as the routine does */
static void sinmom(double box, int npun, int npundim, double xmred, double hbr, double *pr, double *p2r)
{
    double dpi = 2.0 * MW3_PI;
    double hbrxm = 0.5 * hbr * hbr / xmred;
    double ah = box / (double)(npun - 1);
    box = 2.0 * ((double)npun + 1.0) * ah;
    for (int ir = 0; ir < npundim; ir++) { if (pr) pr[ir] = 0.0; p2r[ir] = 0.0; }
    for (int ir = 1; ir <= npun; ir++) {
        double p = dpi * (double)ir / box;
        if (pr) pr[ir - 1] = p;
        p2r[ir - 1] = p * p * hbrxm;
    }
}

/* fftmom (liboctdyn.f:1119-1152) */
static void fftmom(double box, int npun, double *pr)
{
    double dpi = 2.0 * MW3_PI;
    double ah = box / (double)(npun - 1);
    box = ah * (double)npun;
    for (int ir = 1; ir <= npun; ir++) {
        int iii = (ir <= npun / 2) ? ir - 1 : ir - npun - 1;
        pr[ir - 1] = dpi * (double)iii / box;
    }
}

/* eigenvalues of a small symmetric matrix by cyclic Jacobi rotations, ascending */
static void sym_eigvals(int n, double *a /* n*n, destroyed */, double *ev)
{
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0.0;
        for (int p = 0; p < n; p++) for (int q = p + 1; q < n; q++) off += fabs(a[p * n + q]);
        if (off == 0.0) break;
        for (int p = 0; p < n; p++) {
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
    }
    for (int i = 0; i < n; i++) ev[i] = a[i * n + i];
    for (int i = 0; i < n; i++)
        for (int j = i + 1; j < n; j++)
            if (ev[j] < ev[i]) { double t = ev[i]; ev[i] = ev[j]; ev[j] = t; }
}

/* Riccati-Bessel F_l = x j_l(x) and G_l = x y_l(x) (G ~ -cos(x - l pi/2)), the
   open-channel output of BESPH2 (liboctdyn.f:743-835).  G by upward recurrence;
   F upward for x > l, otherwise Miller's downward recurrence normalised to F_0. */
void mw3ref_riccati(int l, double x, double *f, double *g)
{
    double s = sin(x), c = cos(x);
    double g0 = -c, g1 = -c / x - s;
    double gl = g0;
    if (l >= 1) {
        double gm = g0, gc = g1;
        for (int k = 1; k < l; k++) { double gn = (2.0 * k + 1.0) / x * gc - gm; gm = gc; gc = gn; }
        gl = gc;
    }
    *g = gl;
    if (l == 0) { *f = s; return; }
    if (x > (double)l) {
        double fm = s, fc = s / x - c;
        for (int k = 1; k < l; k++) { double fn = (2.0 * k + 1.0) / x * fc - fm; fm = fc; fc = fn; }
        *f = fc;
        return;
    }
    int nstart = l + 40 + (int)x;
    double fp = 0.0, fc = 1e-300, fl = 0.0;
    for (int k = nstart; k >= 1; k--) {
        double fn = (2.0 * k + 1.0) / x * fc - fp;
        fp = fc; fc = fn;
        if (k - 1 == l) fl = fc;
        if (fabs(fc) > 1e250) { fc *= 1e-250; fp *= 1e-250; fl *= 1e-250; }
    }
    /* fc now holds the unnormalised F_0, fp the unnormalised F_1 */
    double scale = (fabs(s) > fabs(s / x - c)) ? s / fc : (s / x - c) / fp;
    *f = fl * scale;
}

/* ---------------------------------------------------------------------- */
/* oracle state                                                            */
/* ---------------------------------------------------------------------- */

struct mw3ref {
    mw3ref_in in;
    int nthreads, dstmode;
    int n1, n2, na, ne, nc, npt;
    int64_t ntot;
    int64_t *offs;            /* [nangu][ncan] flat start (0-based) */
    int *aorder;              /* angle order of the flat vector, 1-based angles */
    /* Tradial */
    int *nopr1, *nopr2;
    double *p2r1, *p2r2;      /* [nangu][npun1], [nangu][npun2] */
    /* kinetic tables */
    double *xj2;              /* [ncan][jang][iang][npun1] */
    double *xl2p;             /* [3][ncan][jang][iang][npun2]   (q+1) */
    int ecor;                 /* electronic Coriolis variant (mod_Hphi_eCoriolis_01y2.f) */
    double *xj2e;             /* [ncan src][ncan dst][jang][iang][npun1], ecor only */
    /* absorption */
    double *absfr1, *absfr2;
    int ir1abs, ir2abs;
    /* propagation state */
    double *psi_km1, *psi_k, *hpsi, *hproc;
    int64_t it;
    /* flux */
    int ir4flux;
    cplx *zar1flux;           /* [npun1] */
    int *ir1flux;             /* [nangu] */
    int nflux;
    int *fl_ang, *fl_can, *fl_r2;   /* flux points */
    int64_t *fl_idx;          /* flat index of each flux point */
    double *potiflux;
    int flux_gate;            /* 1: flux only where E > V(flux point) */
    double *psi0;             /* photodissociation: the initial packet (check's rpaq0) */
    double autocor;           /* <psi0|psi_k> of the last iteration */
    cplx *zcr, *zcdr;         /* [nflux][netot] */
    double *etot, *reacfct, *apaqini, *s2factor;  /* s2factor [nelec][nj][nv][netot] */
    cplx *zck;                /* [netot] */
    int icanref;
    int nj, nv;
    cplx *zs2;                /* [ncan][nj][nv][netot] */
    double *cvj;              /* [ncan][nj][nv] */
    cplx *zfe;                /* [nofe][ntot] */
    dstcache *caches;         /* one per thread */
    struct prodproj *prod;    /* product-state projection (iprod = 2), or NULL */
};

/* the tables of the product-state projection (mod_coortrans01_02.f:21-22, 90-97,
   255-260), 0-based copies; ranges inclusive as in the reference */
typedef struct prodproj {
    int n2p0, n2p1, a0, a1, om0, om1, jp0, jp1, vp0, vp1;
    int32_t *nobcprod;        /* [njp] */
    double *transrgjac;       /* [ntot] */
    double *dtrans;           /* [ncan][nom][nang][n2p] */
    double *prodwf;           /* [nom][njp][nvp][nelec][nang][n2p] */
    double *cvjprod;          /* [nom][njp][nvp] */
    cplx *zs2prod;            /* [nom][njp][nvp][netot] */
} prodproj;

static inline const double *DJ(const mw3ref *r, int iom, int ielec, int j, int iang)
{
    const mw3ref_in *in = &r->in;
    return in->djmmp + ((((size_t)iom * in->nelec + (ielec - 1)) * (in->nangu2 + 1) + j) * in->nangu + (iang - 1));
}
#define DJV(r, iom, ielec, j, iang) (*DJ(r, iom, ielec, j, iang))

static void set_err(char *err, int errlen, const char *msg)
{
    if (err && errlen > 0) { strncpy(err, msg, errlen - 1); err[errlen - 1] = 0; }
}

/* Tradial (mod_Hphi_01y2.f:487-620) */
static void tradial(mw3ref *r)
{
    const mw3ref_in *in = &r->in;
    int na = r->na;
    for (int a = 0; a < na; a++) { r->nopr1[a] = 1; r->nopr2[a] = 1; }
    for (int a = 1; a <= na; a++) {
        int np = in->npunreal[a - 1];
        int ir1min = in->npun1, ir1max = 0;
        for (int ir = 0; ir < np; ir++) {
            int ir1 = in->indr1[(size_t)(a - 1) * in->npuntot + ir];
            if (ir1 < ir1min) ir1min = ir1;
            if (ir1 > ir1max) ir1max = ir1;
        }
        r->nopr1[a - 1] = ir1max - ir1min + 1;
    }
    for (int e = 0; e < in->nelec; e++) {
        for (int a = 0; a < na; a++) {
            int n0 = r->nopr1[a];
            int n1 = noptfft(n0, in->npun1);
            if (n1 < in->npun1min) n1 = in->npun1min;
            r->nopr1[a] = n1;
            if (in->npun1 > 1) {
                double box = (double)(n1 - 1) * in->ah1;
                sinmom(box, n1, in->npun1, in->xm1red, in->hbr, NULL, r->p2r1 + (size_t)a * in->npun1);
            }
            int n2 = in->npun2;
            r->nopr2[a] = n2;
            double box = (double)(n2 - 1) * in->ah2;
            sinmom(box, n2, in->npun2, in->xm2red, in->hbr, NULL, r->p2r2 + (size_t)a * in->npun2);
        }
    }
}

/* angkinj2 (mod_Hphi_01y2.f:166-311), without the Proj_j2_up branch */
static void angkinj2(mw3ref *r)
{
    const mw3ref_in *in = &r->in;
    int na = r->na, n1 = r->n1;
    memset(r->xj2, 0, sizeof(double) * (size_t)r->nc * na * na * n1);
    if (na <= 1) return;
    int jjjmax = (na - 1) * in->inc;
    for (int b = 0; b < r->nc; b++) {
        int ielec = in->nelebas[b], iom = in->iombas[b];
        int iomdi = in->iomdiat[ielec - 1];
        int nojb = in->nojbas[b];
        const int32_t *jb = in->jbas + (size_t)b * na;
        for (int ir1 = 1; ir1 <= n1; ir1++) {
            double r1 = in->rmis1 + (double)(ir1 - 1) * in->ah1;
            for (int k = 0; k < nojb; k++) {
                if (jb[k] > jjjmax) continue;
                double xj = (double)jb[k], xom = (double)iomdi;
                double xkinj = (xj * (xj + 1.0) - xom * xom) * in->hbr * in->hbr * 0.5;
                double yyy = xkinj / (in->xm1red * r1 * r1);
                if (yyy > in->rotcutmax) yyy = in->rotcutmax;
                for (int i = 1; i <= na; i++) {
                    double x1 = DJV(r, iom, ielec, jb[k], i);
                    for (int jang = 1; jang <= na; jang++) {
                        double x2 = DJV(r, iom, ielec, jb[k], jang);
                        size_t o = (((size_t)b * na + (jang - 1)) * na + (i - 1)) * n1 + (ir1 - 1);
                        r->xj2[o] = r->xj2[o] + yyy * x1 * x2;
                    }
                }
            }
        }
    }
}

/* The channel-pair j^2 matrices of the electronic Coriolis variant: angkinj2 of
   mod_Hphi_eCoriolis_01y2.f:186-324 fills xj2(ir1,i,jp,icanp,jcanp) for every
   pair of channels; the diagonal pairs equal the plain xj2 above, and difs reads
   the off-diagonal ones only for equal Omega and |Lambda - Lambda'| = 1
   (:901-911).  Those come from the second branch of its xkinj (:249-258):
   same j at the same basis index k, same sigma, |Lambda - Lambda'| = 1,
   xkinj(k,k) = sqrt(L^2 + L'^2) sqrt(j(j+1) - |L L'|) hbar^2, times sqrt(2)
   when either Lambda is 0; transformed with the source channel's Djmmp on
   both sides (:270-285).  Its third branch (different sigma, equal Lambda)
   fills pairs difs never reads and is not restated. */
static void angkinj2_ecor(mw3ref *r)
{
    const mw3ref_in *in = &r->in;
    int na = r->na, n1 = r->n1, nc = r->nc;
    memset(r->xj2e, 0, sizeof(double) * (size_t)nc * nc * na * na * n1);
    if (na <= 1) return;
    int jjjmax = (na - 1) * in->inc;
    for (int bd = 0; bd < nc; bd++) {                 /* jcanp */
        int jelec = in->nelebas[bd], jom = in->iombas[bd];
        int jomdi = in->iomdiat[jelec - 1];
        for (int b = 0; b < nc; b++) {                /* icanp */
            if (b == bd) continue;
            int ielec = in->nelebas[b], iom = in->iombas[b];
            int iomdi = in->iomdiat[ielec - 1];
            if (iom != jom || in->sigdiat[ielec - 1] != in->sigdiat[jelec - 1]) continue;
            if (abs(jomdi - iomdi) != 1) continue;
            const int32_t *jb = in->jbas + (size_t)b * na, *jbd = in->jbas + (size_t)bd * na;
            int nk = in->nojbas[b] < in->nojbas[bd] ? in->nojbas[b] : in->nojbas[bd];
            for (int ir1 = 1; ir1 <= n1; ir1++) {
                double r1 = in->rmis1 + (double)(ir1 - 1) * in->ah1;
                for (int k = 0; k < nk; k++) {
                    if (jb[k] != jbd[k] || jb[k] > jjjmax) continue;
                    double xj = (double)jb[k];
                    double xlam = sqrt((double)(iomdi * iomdi) + (double)(jomdi * jomdi));
                    double xom = sqrt(xj * (xj + 1) - (double)abs(jomdi * iomdi));
                    double xkinj = xlam * xom * in->hbr * in->hbr;
                    if (jomdi == 0 || iomdi == 0) xkinj = xkinj * sqrt(2.0);
                    double yyy = xkinj / (in->xm1red * r1 * r1);
                    if (yyy > in->rotcutmax) yyy = in->rotcutmax;
                    for (int i = 1; i <= na; i++) {
                        double x1 = DJV(r, iom, ielec, jb[k], i);
                        for (int jang = 1; jang <= na; jang++) {
                            double x2 = DJV(r, iom, ielec, jb[k], jang);
                            size_t o = ((((size_t)b * nc + bd) * na + (jang - 1)) * na + (i - 1)) * n1 + (ir1 - 1);
                            r->xj2e[o] = r->xj2e[o] + yyy * x1 * x2;
                        }
                    }
                }
            }
        }
    }
}

void mw3ref_set_ecoriolis(mw3ref *r, int on)
{
    r->ecor = on != 0;
    free(r->xj2e);
    r->xj2e = NULL;
    if (r->ecor) {
        r->xj2e = (double *)malloc(sizeof(double) * (size_t)r->nc * r->nc * r->na * r->na * r->n1);
        angkinj2_ecor(r);
    }
}

/* l2mat (liboctdyn.f:1944-1990); bfl indexed [iom-iom0][jom-iom0] */
static void l2mat(double *bfl, int nn, double facmass, int iom0, int iom1, int j, int Jtot)
{
    double xj = (double)j;
    for (int iom = iom0; iom <= iom1; iom++)
        for (int jom = iom0; jom <= iom1; jom++) {
            double xk = 0.0;
            if (iom == jom) {
                double x1 = xj * (xj + 1.0);
                double x2 = (double)(Jtot * (Jtot + 1) - 2 * iom * jom);
                xk = (x1 + x2) * facmass;
            } else if (abs(iom - jom) == 1) {
                double x1 = (double)(Jtot * (Jtot + 1) - iom * jom);
                double x2 = xj * (xj + 1.0) - (double)(iom * jom);
                double x12 = sqrt(x1 * x2);
                xk = -x12 * facmass;
                if (iom * jom == 0) xk = xk * sqrt(2.0);
            }
            bfl[(iom - iom0) * nn + (jom - iom0)] = xk;
        }
}

/* bfgridl2mat (mod_Hphi_01y2.f:315-484) */
static void bfgridl2mat(mw3ref *r)
{
    const mw3ref_in *in = &r->in;
    int na = r->na, n2 = r->n2, nc = r->nc;
    memset(r->xl2p, 0, sizeof(double) * 3 * (size_t)nc * na * na * n2);
    double facmass = in->hbr * in->hbr * 0.5 / in->xm2red;
    int maxomg = in->iommax - in->iommin + 1;
    double *bfl = (double *)malloc(sizeof(double) * maxomg * maxomg);
    double *hm = (double *)malloc(sizeof(double) * maxomg * maxomg);
    double *ev = (double *)malloc(sizeof(double) * maxomg);
    double *xl2 = (double *)malloc(sizeof(double) * maxomg * maxomg);
    for (int ielec = 1; ielec <= in->nelec; ielec++) {
        int sigelec = 1;
        if (in->sigdiat[ielec - 1] == -1.0 || in->sigatom[ielec - 1] == -1.0) sigelec = -1;
        for (int j = in->j0; j <= (na - 1) * in->inc; j += in->inc) {
            int iom0 = in->iommin;
            int pj = (in->Jtot % 2) ? -1 : 1;
            if (in->iparity != sigelec * pj && in->iommin == 0) iom0 = 1;
            if (iom0 > j) continue;
            int iom1 = j < in->iommax ? j : in->iommax;
            int nnn = iom1 - iom0 + 1;
            if (nnn <= 0) continue;
            l2mat(bfl, nnn, facmass, iom0, iom1, j, in->Jtot);
            double yylmin, yylmax, yylmean;
            if (nnn > 1) {
                memcpy(hm, bfl, sizeof(double) * nnn * nnn);
                sym_eigvals(nnn, hm, ev);
                yylmin = ev[0]; yylmax = ev[nnn - 1];
                yylmean = 0.5 * (yylmin + yylmax);
            } else {
                yylmin = bfl[0]; yylmax = yylmin; yylmean = yylmin;
            }
            for (int ir2 = 1; ir2 <= n2; ir2++) {
                double r2 = in->rmis2 + (double)(ir2 - 1) * in->ah2;
                double r2eff = r2;
                double emeaneff = yylmean / (r2 * r2);
                if (emeaneff > in->rotcutmax) {
                    double eee = in->rotcutmax;
                    r2eff = sqrt(fabs(yylmean / eee));
                }
                for (int a = 0; a < nnn; a++)
                    for (int c = 0; c < nnn; c++) {
                        double v = 0.0;
                        double bv = bfl[a * nnn + c];
                        if (fabs(bv) > 1e-8 && r2eff > 1e-3) v = bv / (r2eff * r2eff);
                        xl2[a * nnn + c] = v;
                    }
                for (int iom = iom0; iom <= iom1; iom++)
                    for (int jom = iom0; jom <= iom1; jom++) {
                        if (abs(jom - iom) > 1) continue;
                        int iq = (iom == jom) ? 0 : (jom == iom + 1 ? 1 : -1);
                        double yyy = xl2[(iom - iom0) * nnn + (jom - iom0)];
                        for (int b = 0; b < nc; b++) {
                            if (in->nelebas[b] != ielec || in->iombas[b] != jom) continue;
                            for (int iang = 1; iang <= na; iang++) {
                                double x11 = DJV(r, iom, ielec, j, iang);
                                for (int jang = 1; jang <= na; jang++) {
                                    double x22 = DJV(r, jom, ielec, j, jang);
                                    size_t o = ((((size_t)(iq + 1) * nc + b) * na + (jang - 1)) * na + (iang - 1)) * n2 + (ir2 - 1);
                                    r->xl2p[o] = r->xl2p[o] + x11 * x22 * yyy;
                                }
                            }
                        }
                    }
            }
        }
    }
    free(bfl); free(hm); free(ev); free(xl2);
}

/* ini_absorcion (mod_absorcion_01y2.f:28-107) */
static void ini_absorcion(mw3ref *r)
{
    const mw3ref_in *in = &r->in;
    r->ir1abs = in->npun1;
    r->ir2abs = in->npun2;
    for (int ir1 = 1; ir1 <= in->npun1; ir1++) {
        double f1 = 1.0;
        double r1 = (double)(ir1 - 1) * in->ah1 + in->rmis1;
        if (r1 >= in->absr1) {
            if (ir1 < r->ir1abs) r->ir1abs = ir1;
            double delta = (r1 - in->absr1) / (double)in->ninterv1;
            double deltan = powi(delta, in->n1expo);
            double expo = in->absalp1 * deltan;
            f1 = exp(-expo);
        }
        r->absfr1[ir1 - 1] = f1;
    }
    for (int ir2 = 1; ir2 <= in->npun2; ir2++) {
        double f2 = 1.0;
        double r2 = (double)(ir2 - 1) * in->ah2 + in->rmis2;
        if (r2 >= in->absr2) {
            if (ir2 < r->ir2abs) r->ir2abs = ir2;
            double delta = (r2 - in->absr2) / (double)in->ninterv2;
            double deltan = powi(delta, in->n2expo);
            double expo = in->absalp2 * deltan;
            f2 = exp(-expo);
        }
        r->absfr2[ir2 - 1] = f2;
    }
}

/* ini_flux (mod_flux_01y2.f:54-334) and Smatini_col (:392-524) */
static int ini_flux(mw3ref *r, char *err, int errlen)
{
    const mw3ref_in *in = &r->in;
    int n1 = r->n1, na = r->na, nc = r->nc;
    r->nflux = 0;
    if (n1 > 1) {
        double r1flux = in->r1flux_ang;
        r->ir4flux = 0;
        for (int ir1 = 1; ir1 <= n1; ir1++) {
            double r1 = in->rmis1 + (double)(ir1 - 1) * in->ah1;
            if (r1 <= r1flux && ir1 > r->ir4flux) r->ir4flux = ir1;
        }
        double *xpr1 = (double *)malloc(sizeof(double) * n1);
        double box1 = (double)(n1 - 1) * in->ah1;
        fftmom(box1, n1, xpr1);
        for (int m = 1; m <= n1; m++) {
            double delta2r = (double)(r->ir4flux - m) * in->ah1;
            cplx z = {0.0, 0.0};
            for (int k = 1; k <= n1; k++) {
                double xk = xpr1[k - 1];
                cplx a = {0.0, xk};
                cplx e = {cos(xk * delta2r), sin(xk * delta2r)};
                z = cadd(z, cmul(a, e));
            }
            r->zar1flux[m - 1].re = z.re / (double)(2 * n1);
            r->zar1flux[m - 1].im = z.im / (double)(2 * n1);
        }
        free(xpr1);
        for (int a = 0; a < na; a++) r->ir1flux[a] = 0;
        int cnt = 0;
        for (int ia = 0; ia < na; ia++) {
            int iang = r->aorder[ia];
            int np = in->npunreal[iang - 1];
            for (int b = 0; b < nc; b++) {
                for (int ir = 0; ir < np; ir++) {
                    int ir1 = in->indr1[(size_t)(iang - 1) * in->npuntot + ir];
                    double r1 = (double)(ir1 - 1) * in->ah1 + in->rmis1;
                    if (r1 <= r1flux && ir1 > r->ir1flux[iang - 1]) r->ir1flux[iang - 1] = ir1;
                }
                for (int ir = 0; ir < np; ir++)
                    if (in->indr1[(size_t)(iang - 1) * in->npuntot + ir] == r->ir1flux[iang - 1]) cnt++;
            }
        }
        r->nflux = cnt;
        r->fl_ang = (int *)malloc(sizeof(int) * (cnt + 1));
        r->fl_can = (int *)malloc(sizeof(int) * (cnt + 1));
        r->fl_r2 = (int *)malloc(sizeof(int) * (cnt + 1));
        r->potiflux = (double *)malloc(sizeof(double) * (cnt + 1));
        r->fl_idx = (int64_t *)malloc(sizeof(int64_t) * (cnt + 1));
        int f = 0;
        for (int ia = 0; ia < na; ia++) {
            int iang = r->aorder[ia];
            int np = in->npunreal[iang - 1];
            for (int b = 0; b < nc; b++) {
                int ielec = in->nelebas[b];
                for (int ir = 0; ir < np; ir++) {
                    int ir1 = in->indr1[(size_t)(iang - 1) * in->npuntot + ir];
                    if (ir1 == r->ir1flux[iang - 1]) {
                        r->fl_ang[f] = iang;
                        r->fl_can[f] = b;
                        r->fl_r2[f] = in->indr2[(size_t)(iang - 1) * in->npuntot + ir];
                        r->fl_idx[f] = r->offs[(size_t)(iang - 1) * nc + b] + ir;
                        r->potiflux[f] = in->vvv[(((size_t)(ielec - 1) * in->nelec + (ielec - 1)) * na + (iang - 1)) * in->npuntot + ir];
                        f++;
                    }
                }
            }
        }
        r->zcr = (cplx *)calloc((size_t)cnt * in->netot + 1, sizeof(cplx));
        r->zcdr = (cplx *)calloc((size_t)cnt * in->netot + 1, sizeof(cplx));
    }
    /* Smatini: reference channel */
    r->icanref = -1;
    for (int b = 0; b < nc; b++)
        if (in->nelebas[b] == in->ielecref && in->iombas[b] == abs(in->iomref)) r->icanref = b;
    if (r->icanref < 0) { set_err(err, errlen, "icanref can not be set"); return -1; }
    if (in->iphoto < 0 || in->iphoto > 2) { set_err(err, errlen, "iphoto must be 0, 1 or 2"); return -1; }
    int netot = in->netot;
    double etotmin = in->ekinmin, etotmax = in->ekinmax;
    double estep = (etotmax - etotmin) / (double)(netot - 1);
    if (in->iphoto >= 1) {
        /* Smatini_photo (mod_flux_01y2.f:526-581) */
        for (int ie = 0; ie < netot; ie++) {
            r->etot[ie] = etotmin + (double)ie * estep;
            r->apaqini[ie] = 0.0;
            r->reacfct[ie] = 0.25 / MW3_PI / in->xm1reac;
            for (int e = 0; e < in->nelec; e++)
                for (int jj = 0; jj < r->nj; jj++)
                    for (int iv = 0; iv < r->nv; iv++) {
                        double ekinfin = r->etot[ie] - in->ediat[((size_t)e * r->nj + jj) * r->nv + iv];
                        double pfin = ekinfin > 0.0 ? sqrt(ekinfin * in->xm2reac * 2.0 / in->hbr / in->hbr) : 0.0;
                        r->s2factor[(((size_t)e * r->nj + jj) * r->nv + iv) * netot + ie] =
                            4.0 * pfin / (MW3_PI * in->xm2reac);
                    }
        }
        return 0;
    }
    /* Smatini_col */
    const int npunt = 1000;
    double *rg = (double *)malloc(sizeof(double) * npunt);
    double ahgauss = (in->rfin2 - in->rmis2) / (double)(npunt - 1);
    for (int ir2 = 1; ir2 <= npunt; ir2++) {
        double r2 = in->rmis2 + (double)(ir2 - 1) * ahgauss;
        double g = cos((r2 - in->rcolini) * in->xk0) * sqrt(2.0);
        double xr2 = g * in->factor0 * exp(-(r2 - in->rcolini) * (r2 - in->rcolini) / in->alpha0 / in->alpha0);
        rg[ir2 - 1] = xr2 / sqrt(2.0);
    }
    double pepe = (double)(in->il0 * (in->il0 + 1));
    double rr = in->rcolini + 1.0;
    double erot = in->hbr * in->hbr * pepe * 0.5 / (rr * rr * in->xmasa0);
    int nj = r->nj, nv = r->nv;
    for (int ie = 0; ie < netot; ie++) {
        r->etot[ie] = etotmin + (double)ie * estep;
        double ekinini = r->etot[ie];
        double paqini = 0.0, pini = 0.0;
        if (ekinini > 0.0 && ekinini > erot) {
            pini = sqrt(ekinini * in->xmasa0 * 2.0 / in->hbr / in->hbr);
            cplx zfft = {0.0, 0.0};
            for (int ir2 = 1; ir2 <= npunt; ir2++) {
                double rx = in->rmis2 + (double)(ir2 - 1) * ahgauss;
                double arg = rx * pini, fb, gb;
                mw3ref_riccati(in->il0, arg, &fb, &gb);
                if (fabs(fb) > 1e-20) {
                    zfft.re += rg[ir2 - 1] * (-gb);
                    zfft.im += rg[ir2 - 1] * fb;
                }
            }
            zfft.re = zfft.re * ahgauss / 2.0 / MW3_PI;
            zfft.im = zfft.im * ahgauss / 2.0 / MW3_PI;
            paqini = zfft.re * zfft.re + zfft.im * zfft.im;
        }
        r->apaqini[ie] = paqini;
        for (int e = 0; e < in->nelec; e++)
            for (int jj = 0; jj < nj; jj++)
                for (int iv = 0; iv < nv; iv++) {
                    double ekinfin = r->etot[ie] - in->ediat[((size_t)e * nj + jj) * nv + iv];
                    double pfin = ekinfin > 0.0 ? sqrt(ekinfin * in->xm2reac * 2.0 / in->hbr / in->hbr) : 0.0;
                    double v = (paqini < 1e-10) ? 0.0
                        : in->hbr * in->hbr * pfin * pini / (2.0 * paqini) / in->xm2reac / in->xmasa0;
                    r->s2factor[(((size_t)e * nj + jj) * nv + iv) * netot + ie] = v;
                }
        r->reacfct[ie] = (paqini < 1e-10) ? 0.0
            : in->hbr * in->hbr * pini / paqini / in->xmasa0 / in->xm1reac / 4.0 / MW3_PI / MW3_PI;
    }
    free(rg);
    return 0;
}

/* ---------------------------------------------------------------------- */

mw3ref *mw3ref_create(const mw3ref_in *in, char *err, int errlen)
{
    if (in->proj_j2_up != 0) { set_err(err, errlen, "Proj_j2_up != 0 is not restated"); return NULL; }
    if (in->npun1min > in->npun1) { set_err(err, errlen, "npun1min > npun1"); return NULL; }
    for (int a = 0; a < in->nangu; a++)
        if (in->npunreal[a] <= 0) { set_err(err, errlen, "angle without stored points"); return NULL; }
    mw3ref *r = (mw3ref *)calloc(1, sizeof(mw3ref));
    if (r) r->flux_gate = 1;
    r->in = *in;
    r->nthreads = 1;
    r->n1 = in->npun1; r->n2 = in->npun2; r->na = in->nangu; r->ne = in->nelec; r->nc = in->ncan;
    r->npt = in->npuntot;
    int na = r->na, nc = r->nc;
    r->aorder = (int *)malloc(sizeof(int) * na);
    for (int ia = 0; ia < na; ia++) r->aorder[ia] = na - ia;          /* indangreal for nproc=1 */
    r->offs = (int64_t *)malloc(sizeof(int64_t) * na * nc);
    int64_t cnt = 0;
    for (int ia = 0; ia < na; ia++) {
        int iang = r->aorder[ia];
        for (int b = 0; b < nc; b++) { r->offs[(size_t)(iang - 1) * nc + b] = cnt; cnt += in->npunreal[iang - 1]; }
    }
    r->ntot = cnt;
    r->nopr1 = (int *)calloc(na, sizeof(int));
    r->nopr2 = (int *)calloc(na, sizeof(int));
    r->p2r1 = (double *)calloc((size_t)na * r->n1, sizeof(double));
    r->p2r2 = (double *)calloc((size_t)na * r->n2, sizeof(double));
    tradial(r);
    for (int a = 0; a < na; a++)
        if (r->nopr1[a] > r->n1) { set_err(err, errlen, "nopr1 > npun1"); mw3ref_destroy(r); return NULL; }
    r->xj2 = (double *)malloc(sizeof(double) * (size_t)nc * na * na * r->n1);
    r->xl2p = (double *)malloc(sizeof(double) * 3 * (size_t)nc * na * na * r->n2);
    angkinj2(r);
    bfgridl2mat(r);
    r->absfr1 = (double *)malloc(sizeof(double) * r->n1);
    r->absfr2 = (double *)malloc(sizeof(double) * r->n2);
    ini_absorcion(r);
    r->psi_km1 = (double *)calloc(cnt + 1, sizeof(double));
    r->psi_k = (double *)calloc(cnt + 1, sizeof(double));
    r->hpsi = (double *)calloc(cnt + 1, sizeof(double));
    r->hproc = (double *)calloc(cnt + 1, sizeof(double));
    r->zar1flux = (cplx *)calloc(r->n1, sizeof(cplx));
    r->ir1flux = (int *)calloc(na, sizeof(int));
    r->nj = in->jmax - in->jini + 1;
    r->nv = in->nvmax - in->nvini + 1;
    r->etot = (double *)calloc(in->netot, sizeof(double));
    r->reacfct = (double *)calloc(in->netot, sizeof(double));
    r->apaqini = (double *)calloc(in->netot, sizeof(double));
    r->s2factor = (double *)calloc((size_t)in->nelec * r->nj * r->nv * in->netot, sizeof(double));
    r->zck = (cplx *)calloc(in->netot, sizeof(cplx));
    r->zs2 = (cplx *)calloc((size_t)nc * r->nj * r->nv * in->netot, sizeof(cplx));
    r->cvj = (double *)calloc((size_t)nc * r->nj * r->nv, sizeof(double));
    if (in->nofe > 0) r->zfe = (cplx *)calloc((size_t)in->nofe * cnt, sizeof(cplx));
    if (ini_flux(r, err, errlen)) { mw3ref_destroy(r); return NULL; }
    r->caches = (dstcache *)calloc(256, sizeof(dstcache));
    return r;
}

void mw3ref_destroy(mw3ref *r)
{
    if (!r) return;
    if (r->caches) { for (int t = 0; t < 256; t++) plan_free(r->caches[t].plans); free(r->caches); }
    free(r->aorder); free(r->offs); free(r->nopr1); free(r->nopr2); free(r->p2r1); free(r->p2r2);
    free(r->xj2); free(r->xl2p); free(r->xj2e); free(r->absfr1); free(r->absfr2);
    free(r->psi_km1); free(r->psi_k); free(r->hpsi); free(r->hproc);
    free(r->psi0);
    free(r->zar1flux); free(r->ir1flux); free(r->fl_ang); free(r->fl_can); free(r->fl_r2); free(r->fl_idx); free(r->potiflux);
    free(r->zcr); free(r->zcdr); free(r->etot); free(r->reacfct); free(r->apaqini); free(r->s2factor);
    free(r->zck); free(r->zs2); free(r->cvj); free(r->zfe);
    if (r->prod) {
        free(r->prod->nobcprod); free(r->prod->transrgjac); free(r->prod->dtrans); free(r->prod->prodwf);
        free(r->prod->cvjprod); free(r->prod->zs2prod); free(r->prod);
    }
    free(r);
}

int64_t mw3ref_ntot(const mw3ref *r) { return r->ntot; }
void mw3ref_set_threads(mw3ref *r, int n) { r->nthreads = n < 1 ? 1 : (n > 256 ? 256 : n); }
void mw3ref_set_dst_mode(mw3ref *r, int mode) { r->dstmode = mode; }

/* totalflux_k's energy test E > V(flux point) (mod_flux_01y2.f:640): on as in
   the shipped source, or off as in the earlier form that made the shipped
   H + HD run (every energy takes every flux point) */
void mw3ref_set_flux_gate(mw3ref *r, int on) { r->flux_gate = on; }

/* T, V and angular contributions of one source (block, angle) pair: the body of
   the jangp loop of difs (mod_Hphi_01y2.f:748-902).  hrec/hproc are the
   rHpaqrec / rHpaqproc(:,1) accumulators. */
static void difs_source(mw3ref *r, int b, int jang, const double *psi, double *hrec, double *hproc,
                        double *raux, double *rphi0, double *auxr, double *line, double *line2,
                        cplx *buf, cplx *work, dstcache *dc)
{
    const mw3ref_in *in = &r->in;
    int n1 = r->n1, n2 = r->n2, na = r->na, nc = r->nc;
    int ielec = in->nelebas[b], iom = in->iombas[b];
    size_t rect = (size_t)n1 * n2;
    memset(raux, 0, sizeof(double) * rect);
    memset(rphi0, 0, sizeof(double) * rect);
    int np = in->npunreal[jang - 1];
    const int32_t *i1 = in->indr1 + (size_t)(jang - 1) * in->npuntot;
    const int32_t *i2 = in->indr2 + (size_t)(jang - 1) * in->npuntot;
    int64_t i0 = r->offs[(size_t)(jang - 1) * nc + b];
    /* raux(ir2,ir1) is column-major: element (ir2,ir1) at (ir1-1)*n2 + ir2-1 */
    for (int ir = 0; ir < np; ir++) {
        size_t o = (size_t)(i1[ir] - 1) * n2 + (i2[ir] - 1);
        raux[o] = psi[i0 + ir];
        rphi0[o] = raux[o];
    }
    int nn2 = r->nopr2[jang - 1], nn1 = r->nopr1[jang - 1];
    double divi = 4.0 * (double)(nn1 + 1) * (double)(nn2 + 1);
    divi = 1.0 / divi;
    /* auxR(iii), iii = nn2*(ir1-1)+ir2: column-major (nn2, nn1) */
    for (int ir1 = 0; ir1 < nn1; ir1++)
        for (int ir2 = 0; ir2 < nn2; ir2++) auxr[(size_t)ir1 * nn2 + ir2] = raux[(size_t)ir1 * n2 + ir2];
    for (int pass = 0; pass < 2; pass++) {
        /* 2-D RODFT00: along ir2 (contiguous) then along ir1 */
        if (r->dstmode == 1) {
            for (int ir1 = 0; ir1 < nn1; ir1++) {
                dst1_direct(nn2, auxr + (size_t)ir1 * nn2, line);
                memcpy(auxr + (size_t)ir1 * nn2, line, sizeof(double) * nn2);
            }
            for (int ir2 = 0; ir2 < nn2; ir2++) {
                for (int ir1 = 0; ir1 < nn1; ir1++) line2[ir1] = auxr[(size_t)ir1 * nn2 + ir2];
                dst1_direct(nn1, line2, line);
                for (int ir1 = 0; ir1 < nn1; ir1++) auxr[(size_t)ir1 * nn2 + ir2] = line[ir1];
            }
        } else {
            for (int ir1 = 0; ir1 < nn1; ir1 += 2) {
                double *xa = auxr + (size_t)ir1 * nn2;
                double *xb = (ir1 + 1 < nn1) ? auxr + (size_t)(ir1 + 1) * nn2 : NULL;
                dst1_pair_fft(dc, nn2, xa, xb, line, line2, buf, work);
                memcpy(xa, line, sizeof(double) * nn2);
                if (xb) memcpy(xb, line2, sizeof(double) * nn2);
            }
            double *ca = line, *cb = line + n1, *oa = line2, *ob = line2 + n1;
            for (int ir2 = 0; ir2 < nn2; ir2 += 2) {
                int two = (ir2 + 1 < nn2);
                for (int ir1 = 0; ir1 < nn1; ir1++) {
                    ca[ir1] = auxr[(size_t)ir1 * nn2 + ir2];
                    if (two) cb[ir1] = auxr[(size_t)ir1 * nn2 + ir2 + 1];
                }
                dst1_pair_fft(dc, nn1, ca, two ? cb : NULL, oa, two ? ob : NULL, buf, work);
                for (int ir1 = 0; ir1 < nn1; ir1++) {
                    auxr[(size_t)ir1 * nn2 + ir2] = oa[ir1];
                    if (two) auxr[(size_t)ir1 * nn2 + ir2 + 1] = ob[ir1];
                }
            }
        }
        if (pass == 0) {
            const double *p1 = r->p2r1 + (size_t)(jang - 1) * n1;
            const double *p2 = r->p2r2 + (size_t)(jang - 1) * n2;
            for (int ir1 = 0; ir1 < nn1; ir1++)
                for (int ir2 = 0; ir2 < nn2; ir2++) {
                    double ekin = p1[ir1] + p2[ir2];
                    if (ekin > in->radcutmax) ekin = in->radcutmax;
                    size_t o = (size_t)ir1 * nn2 + ir2;
                    auxr[o] = auxr[o] * ekin * divi;
                }
        }
    }
    for (int ir1 = 0; ir1 < nn1; ir1++)
        for (int ir2 = 0; ir2 < nn2; ir2++) raux[(size_t)ir1 * n2 + ir2] = auxr[(size_t)ir1 * nn2 + ir2];
    for (int ir = 0; ir < np; ir++) {
        size_t o = (size_t)(i1[ir] - 1) * n2 + (i2[ir] - 1);
        hrec[i0 + ir] = hrec[i0 + ir] + raux[o];
    }
    /* V part (:838-853) */
    for (int b2 = 0; b2 < nc; b2++) {
        if (in->iombas[b2] != iom) continue;
        int ielec2 = in->nelebas[b2];
        int64_t j0 = r->offs[(size_t)(jang - 1) * nc + b2];
        const double *v = in->vvv + (((size_t)(ielec2 - 1) * in->nelec + (ielec - 1)) * na + (jang - 1)) * in->npuntot;
        for (int ir = 0; ir < np; ir++) {
            size_t o = (size_t)(i1[ir] - 1) * n2 + (i2[ir] - 1);
            hrec[j0 + ir] = hrec[j0 + ir] + rphi0[o] * v[ir];
        }
    }
    /* j^2 + l^2 (:859-902), single process: ncouproc = 1 */
    for (int ia = 0; ia < na; ia++) {
        int iang = r->aorder[ia];
        int npi = in->npunreal[iang - 1];
        const int32_t *t1 = in->indr1 + (size_t)(iang - 1) * in->npuntot;
        const int32_t *t2 = in->indr2 + (size_t)(iang - 1) * in->npuntot;
        for (int b2 = 0; b2 < nc; b2++) {
            int iom2 = in->iombas[b2], ielec2 = in->nelebas[b2];
            int64_t j0 = r->offs[(size_t)(iang - 1) * nc + b2];
            if (ielec != ielec2) {
                /* electronic Coriolis coupling (mod_Hphi_eCoriolis_01y2.f:901-911) */
                if (r->ecor && iom == iom2 && abs(in->iomdiat[ielec - 1] - in->iomdiat[ielec2 - 1]) == 1) {
                    const double *xj = r->xj2e + ((((size_t)b * nc + b2) * na + (jang - 1)) * na + (iang - 1)) * n1;
                    for (int ir = 0; ir < npi; ir++) {
                        int ir1 = t1[ir], ir2 = t2[ir];
                        hproc[j0 + ir] = hproc[j0 + ir] + rphi0[(size_t)(ir1 - 1) * n2 + (ir2 - 1)] * xj[ir1 - 1];
                    }
                }
                continue;
            }
            if (iom == iom2) {
                const double *xj = r->xj2 + (((size_t)b * na + (jang - 1)) * na + (iang - 1)) * n1;
                const double *xl = r->xl2p + ((((size_t)1 * nc + b) * na + (jang - 1)) * na + (iang - 1)) * n2;
                for (int ir = 0; ir < npi; ir++) {
                    int ir1 = t1[ir], ir2 = t2[ir];
                    hproc[j0 + ir] = hproc[j0 + ir] + rphi0[(size_t)(ir1 - 1) * n2 + (ir2 - 1)] * (xj[ir1 - 1] + xl[ir2 - 1]);
                }
            } else if (iom == iom2 + 1 || iom == iom2 - 1) {
                int q = (iom == iom2 + 1) ? 1 : -1;
                const double *xl = r->xl2p + ((((size_t)(q + 1) * nc + b) * na + (jang - 1)) * na + (iang - 1)) * n2;
                for (int ir = 0; ir < npi; ir++) {
                    int ir1 = t1[ir], ir2 = t2[ir];
                    hproc[j0 + ir] = hproc[j0 + ir] + rphi0[(size_t)(ir1 - 1) * n2 + (ir2 - 1)] * xl[ir2 - 1];
                }
            }
        }
    }
}

static void difs(mw3ref *r, const double *psi, double *h)
{
    int64_t n = r->ntot;
    int nt = r->nthreads;
    int n1 = r->n1, n2 = r->n2, na = r->na, nc = r->nc;
    size_t rect = (size_t)n1 * n2;
    int nmax = n1 > n2 ? n1 : n2;
    int mmax = 1; while (mmax < 4 * (nmax + 1)) mmax <<= 1;
    if (nt <= 1) {
        memset(h, 0, sizeof(double) * n);
        memset(r->hproc, 0, sizeof(double) * n);
        double *raux = (double *)malloc(sizeof(double) * rect * 3);
        double *line = (double *)malloc(sizeof(double) * 4 * nmax), *line2 = (double *)malloc(sizeof(double) * 4 * nmax);
        cplx *buf = (cplx *)malloc(sizeof(cplx) * mmax), *work = (cplx *)malloc(sizeof(cplx) * mmax);
        for (int b = 0; b < nc; b++)
            for (int ia = 0; ia < na; ia++)
                difs_source(r, b, r->aorder[ia], psi, h, r->hproc, raux, raux + rect, raux + 2 * rect,
                            line, line2, buf, work, &r->caches[0]);
        for (int64_t i = 0; i < n; i++) h[i] = h[i] + r->hproc[i];
        free(raux); free(line); free(line2); free(buf); free(work);
        return;
    }
    /* threaded over source angles with private accumulators, as the reference's
       OpenMP region does with its reduction(+:rHpaqrec,rHpaqproc) */
    double *acc = (double *)calloc((size_t)nt * 2 * n, sizeof(double));
#pragma omp parallel num_threads(nt)
    {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
        double *hr = acc + (size_t)t * 2 * n, *hp = hr + n;
        double *raux = (double *)malloc(sizeof(double) * rect * 3);
        double *line = (double *)malloc(sizeof(double) * 4 * nmax), *line2 = (double *)malloc(sizeof(double) * 4 * nmax);
        cplx *buf = (cplx *)malloc(sizeof(cplx) * mmax), *work = (cplx *)malloc(sizeof(cplx) * mmax);
        for (int b = 0; b < nc; b++) {
#pragma omp for schedule(dynamic)
            for (int ia = 0; ia < na; ia++)
                difs_source(r, b, r->aorder[ia], psi, hr, hp, raux, raux + rect, raux + 2 * rect,
                            line, line2, buf, work, &r->caches[t]);
        }
        free(raux); free(line); free(line2); free(buf); free(work);
#pragma omp barrier
#pragma omp for schedule(static)
        for (int64_t i = 0; i < n; i++) {
            double s = 0.0, p = 0.0;
            for (int q = 0; q < nt; q++) { s += acc[(size_t)q * 2 * n + i]; p += acc[(size_t)q * 2 * n + n + i]; }
            h[i] = s + p;
        }
    }
    free(acc);
}

int mw3ref_hphi(mw3ref *r, const double *psi, double *hpsi)
{
    difs(r, psi, hpsi);
    return 0;
}

int mw3ref_coefecheby(const mw3ref *r, int64_t k, double *ck)
{
    const mw3ref_in *in = &r->in;
    double d = (k == 0) ? 1.0 : 2.0;
    double zfactor = d * in->hbr / in->delta2;
    for (int ie = 0; ie < in->netot; ie++) {
        double E = r->etot[ie];
        double Es = (E - in->emindlt) / in->delta2;
        double expo = -(double)k * acos(Es);
        double deno = sqrt(1.0 - Es * Es);
        ck[2 * ie] = zfactor * cos(expo) / deno;
        ck[2 * ie + 1] = zfactor * sin(expo) / deno;
    }
    return 0;
}

/* totalflux_k (mod_flux_01y2.f:585-660) */
static void totalflux_k(mw3ref *r, int64_t k)
{
    const mw3ref_in *in = &r->in;
    int n2 = r->n2, na = r->na, nc = r->nc, netot = in->netot;
    cplx *zf = (cplx *)calloc((size_t)n2 * na * nc, sizeof(cplx));   /* zfR1flux(ir2, iang, b) */
    for (int ia = 0; ia < na; ia++) {
        int iang = r->aorder[ia];
        int np = in->npunreal[iang - 1];
        for (int b = 0; b < nc; b++) {
            int64_t i0 = r->offs[(size_t)(iang - 1) * nc + b];
            for (int ir = 0; ir < np; ir++) {
                int ir1 = in->indr1[(size_t)(iang - 1) * in->npuntot + ir];
                int ir2 = in->indr2[(size_t)(iang - 1) * in->npuntot + ir];
                cplx a = r->zar1flux[ir1 - 1];
                size_t o = ((size_t)b * na + (iang - 1)) * n2 + (ir2 - 1);
                double p = r->psi_k[i0 + ir];
                zf[o].re = zf[o].re + (a.re * p - a.im * 0.0);
                zf[o].im = zf[o].im + (a.re * 0.0 + a.im * p);
            }
        }
    }
    for (int f = 0; f < r->nflux; f++) {
        int iang = r->fl_ang[f], b = r->fl_can[f], ir2 = r->fl_r2[f];
        /* zR(ir2): psi at (ir1flux, ir2); zdR(ir2) = zfR1flux(ir2,iang,b) */
        double zr = r->psi_k[r->fl_idx[f]];
        cplx zd = zf[((size_t)b * na + (iang - 1)) * n2 + (ir2 - 1)];
        for (int ie = 0; ie < netot; ie++) {
            cplx ze = r->zck[ie];
            if (in->iphoto == 0 && in->iprod == 1 && k < in->kminelastic) { ze.re = 0; ze.im = 0; }
            if (!r->flux_gate || r->etot[ie] > r->potiflux[f]) {
                cplx *c = &r->zcr[(size_t)f * netot + ie], *d = &r->zcdr[(size_t)f * netot + ie];
                c->re = c->re + (ze.re * zr - ze.im * 0.0);
                c->im = c->im + (ze.re * 0.0 + ze.im * zr);
                cplx m = cmul(ze, zd);
                d->re = d->re + m.re;
                d->im = d->im + m.im;
            }
        }
    }
    free(zf);
}

/* Cvjflux_k (mod_flux_01y2.f:663-775) */
static void cvjflux_k(mw3ref *r, int64_t k)
{
    const mw3ref_in *in = &r->in;
    int n1 = r->n1, na = r->na, nc = r->nc, nj = r->nj, nv = r->nv, netot = in->netot;
    double *funreac = (double *)calloc((size_t)na * n1 * nc, sizeof(double));   /* [b][iang][ir1] */
    double *rpopi = (double *)calloc((size_t)nc * nj * nv, sizeof(double));
    double sah2 = sqrt(in->ah2);
    for (int ia = 0; ia < na; ia++) {
        int iang = r->aorder[ia];
        int np = in->npunreal[iang - 1];
        for (int b = 0; b < nc; b++) {
            int64_t i0 = r->offs[(size_t)(iang - 1) * nc + b];
            for (int ir = 0; ir < np; ir++) {
                if (in->indr2[(size_t)(iang - 1) * in->npuntot + ir] == r->ir2abs) {
                    int ir1 = in->indr1[(size_t)(iang - 1) * in->npuntot + ir];
                    funreac[((size_t)b * na + (iang - 1)) * n1 + (ir1 - 1)] = r->psi_k[i0 + ir] / sah2;
                }
            }
        }
    }
    for (int b = 0; b < nc; b++) {
        int ielec = in->nelebas[b], iom = in->iombas[b];
        for (int ir1 = 1; ir1 <= n1; ir1++) {
            for (int j = in->j00[b]; j <= in->jmax; j += in->inc) {
                double xj = 0.0;
                for (int ia = 0; ia < na; ia++) {
                    int iang = r->aorder[ia];
                    double rori = funreac[((size_t)b * na + (iang - 1)) * n1 + (ir1 - 1)];
                    xj = xj + rori * DJV(r, iom, ielec, j, iang);
                }
                int nob = in->nobc[(size_t)(ielec - 1) * nj + (j - in->jini)];
                int maxnv = in->nvmax < nob ? in->nvmax : nob;
                for (int iv = in->nvini; iv <= maxnv; iv++) {
                    size_t o = ((size_t)b * nj + (j - in->jini)) * nv + (iv - in->nvini);
                    const double *fdv = in->fd + ((((size_t)(ielec - 1) * nj + (j - in->jini)) * nv + (iv - in->nvini)) * n1);
                    rpopi[o] = rpopi[o] + xj * fdv[ir1 - 1];
                }
            }
        }
    }
    memset(r->cvj, 0, sizeof(double) * (size_t)nc * nj * nv);
    for (int b = 0; b < nc; b++) {
        int ielec = in->nelebas[b];
        for (int j = in->j00[b]; j <= in->jmax; j += in->inc) {
            int nob = in->nobc[(size_t)(ielec - 1) * nj + (j - in->jini)];
            int maxnv = in->nvmax < nob ? in->nvmax : nob;
            for (int iv = in->nvini; iv <= maxnv; iv++) {
                size_t o = ((size_t)b * nj + (j - in->jini)) * nv + (iv - in->nvini);
                r->cvj[o] = rpopi[o];
            }
        }
    }
    for (int b = 0; b < nc; b++) {
        int ielec = in->nelebas[b];
        for (int j = in->j00[b]; j <= in->jmax; j += in->inc) {
            int nob = in->nobc[(size_t)(ielec - 1) * nj + (j - in->jini)];
            int maxnv = in->nvmax < nob ? in->nvmax : nob;
            for (int iv = in->nvini; iv <= maxnv; iv++) {
                int ifail = 0;
                if (in->iomref >= 0) {
                    if (b == r->icanref && iv == in->nvref && j == in->jref)
                        if (in->iprod != 1 && in->iphoto == 0 && k < in->kminelastic) ifail = 1;
                } else {
                    if (iv == in->nvref && j == in->jref)
                        if (in->iprod != 1 && in->iphoto == 0 && k < in->kminelastic) ifail = 1;
                }
                if (ifail) continue;
                size_t o = ((size_t)b * nj + (j - in->jini)) * nv + (iv - in->nvini);
                double z = r->cvj[o];
                for (int ie = 0; ie < netot; ie++) {
                    cplx *s = &r->zs2[o * netot + ie];
                    cplx ck = r->zck[ie];
                    s->re = s->re + (z * ck.re - 0.0 * ck.im);
                    s->im = s->im + (z * ck.im + 0.0 * ck.re);
                }
            }
        }
    }
    free(funreac); free(rpopi);
}

/* funE (mod_PsiE_01y2.f:92-123) */
static void fune(mw3ref *r, int64_t k)
{
    const mw3ref_in *in = &r->in;
    double d = (k == 0) ? 1.0 : 2.0;
    double zfactor = d * in->hbr / in->delta2;
    for (int e = 0; e < in->nofe; e++) {
        double Es = (in->efe[e] - in->emindlt) / in->delta2;
        double expo = -(double)k * acos(Es);
        double deno = sqrt(1.0 - Es * Es);
        cplx ck = {zfactor * cos(expo) / deno, zfactor * sin(expo) / deno};
        cplx *z = r->zfe + (size_t)e * r->ntot;
        for (int64_t i = 0; i < r->ntot; i++) {
            z[i].re = z[i].re + ck.re * r->psi_k[i];
            z[i].im = z[i].im + ck.im * r->psi_k[i];
        }
    }
}

/* prodpaq (mod_coortrans01_02.f:694-788): psi_k binned on (block, angle, R)
   with the weights transRgjac over the projection's R and angle ranges, then
   Cvjprod(v,j,Omega) = sum over blocks and (angle, R) of
   prodwf(R,angle,e,v,j,Omega) funprod(R,angle,block) dtrans(R,angle,Omega,block) */
static void prodpaq(mw3ref *r)
{
    const mw3ref_in *in = &r->in;
    prodproj *p = r->prod;
    const int nc = r->nc, n2p = p->n2p1 - p->n2p0 + 1, nang = p->a1 - p->a0 + 1;
    const int njp = p->jp1 - p->jp0 + 1, nvp = p->vp1 - p->vp0 + 1;
    double *fun = (double *)calloc((size_t)nc * nang * n2p, sizeof(double));
    double *aux = (double *)malloc(sizeof(double) * r->n2);
    double *aux2 = (double *)malloc(sizeof(double) * (size_t)nang * n2p);
    for (int b = 0; b < nc; b++)
        for (int iang = p->a0; iang <= p->a1; iang++) {
            for (int k = 0; k < r->n2; k++) aux[k] = 0.0;
            int np = in->npunreal[iang - 1];
            int64_t i0 = r->offs[(size_t)(iang - 1) * nc + b];
            for (int ir = 0; ir < np; ir++) {
                int ir2 = in->indr2[(size_t)(iang - 1) * in->npuntot + ir];
                aux[ir2 - 1] = aux[ir2 - 1] + p->transrgjac[i0 + ir] * r->psi_k[i0 + ir];
            }
            for (int ir2 = p->n2p0; ir2 <= p->n2p1; ir2++)
                fun[((size_t)b * nang + (iang - p->a0)) * n2p + (ir2 - p->n2p0)] = aux[ir2 - 1];
        }
    memset(p->cvjprod, 0, sizeof(double) * (size_t)(p->om1 - p->om0 + 1) * njp * nvp);
    for (int b = 0; b < nc; b++) {
        int ielec = in->nelebas[b];
        for (int iom = p->om0; iom <= p->om1; iom++) {
            const int o = iom - p->om0;
            int jinip = p->jp0 > iom ? p->jp0 : iom;
            const double *dt = p->dtrans + (((size_t)b * (p->om1 - p->om0 + 1) + o) * nang) * n2p;
            const double *fb = fun + (size_t)b * nang * n2p;
            for (size_t k = 0; k < (size_t)nang * n2p; k++) aux2[k] = fb[k] * dt[k];
            for (int j = jinip; j <= p->jp1; j++)
                for (int iv = p->vp0; iv <= p->nobcprod[j - p->jp0]; iv++) {
                    const double *wf =
                        p->prodwf + ((((size_t)o * njp + (j - p->jp0)) * nvp + (iv - p->vp0)) * in->nelec + (ielec - 1)) *
                                        nang * n2p;
                    double x = 0.0;
                    for (size_t k = 0; k < (size_t)nang * n2p; k++) x = x + wf[k] * aux2[k];
                    double *c = &p->cvjprod[((size_t)o * njp + (j - p->jp0)) * nvp + (iv - p->vp0)];
                    *c = *c + x;
                }
        }
    }
    free(fun); free(aux); free(aux2);
}

/* prodcvj (mod_coortrans01_02.f:791-825): zS2prod(E,v,j,Omega) += Cvjprod C_k(E) */
static void prodcvj(mw3ref *r)
{
    prodproj *p = r->prod;
    const int netot = r->in.netot, njp = p->jp1 - p->jp0 + 1, nvp = p->vp1 - p->vp0 + 1;
    for (int iom = p->om0; iom <= p->om1; iom++) {
        int jinip = p->jp0 > iom ? p->jp0 : iom;
        for (int j = jinip; j <= p->jp1; j++)
            for (int iv = p->vp0; iv <= p->nobcprod[j - p->jp0]; iv++) {
                size_t o = ((size_t)(iom - p->om0) * njp + (j - p->jp0)) * nvp + (iv - p->vp0);
                double z = p->cvjprod[o];
                for (int ie = 0; ie < netot; ie++) {
                    cplx *s = &p->zs2prod[o * netot + ie];
                    cplx ck = r->zck[ie];
                    s->re = s->re + (z * ck.re - 0.0 * ck.im);
                    s->im = s->im + (z * ck.im + 0.0 * ck.re);
                }
            }
    }
}

int mw3ref_set_product(mw3ref *r, int n2prod0, int n2prod1, int nangproj0, int nangproj1, int iomminprod,
                       int iommaxprod, int jiniprod, int jmaxprod, int nviniprod, int nvmaxprod,
                       const int32_t *nobcprod, const double *transrgjac, const double *dtrans, const double *prodwf)
{
    if (n2prod0 < 1 || n2prod1 > r->n2 || n2prod1 < n2prod0 || nangproj0 < 1 || nangproj1 > r->na ||
        nangproj1 < nangproj0 || iommaxprod < iomminprod || jmaxprod < jiniprod || nvmaxprod < nviniprod)
        return 1;
    for (int j = jiniprod; j <= jmaxprod; j++)
        if (nobcprod[j - jiniprod] > nvmaxprod) return 1;
    prodproj *p = (prodproj *)calloc(1, sizeof(prodproj));
    p->n2p0 = n2prod0; p->n2p1 = n2prod1; p->a0 = nangproj0; p->a1 = nangproj1;
    p->om0 = iomminprod; p->om1 = iommaxprod; p->jp0 = jiniprod; p->jp1 = jmaxprod;
    p->vp0 = nviniprod; p->vp1 = nvmaxprod;
    size_t n2p = n2prod1 - n2prod0 + 1, nang = nangproj1 - nangproj0 + 1, nom = iommaxprod - iomminprod + 1;
    size_t njp = jmaxprod - jiniprod + 1, nvp = nvmaxprod - nviniprod + 1;
    size_t ndt = (size_t)r->nc * nom * nang * n2p, nwf = nom * njp * nvp * r->in.nelec * nang * n2p;
    p->nobcprod = (int32_t *)malloc(sizeof(int32_t) * njp);
    memcpy(p->nobcprod, nobcprod, sizeof(int32_t) * njp);
    p->transrgjac = (double *)malloc(sizeof(double) * r->ntot);
    memcpy(p->transrgjac, transrgjac, sizeof(double) * r->ntot);
    p->dtrans = (double *)malloc(sizeof(double) * ndt);
    memcpy(p->dtrans, dtrans, sizeof(double) * ndt);
    p->prodwf = (double *)malloc(sizeof(double) * nwf);
    memcpy(p->prodwf, prodwf, sizeof(double) * nwf);
    p->cvjprod = (double *)calloc(nom * njp * nvp, sizeof(double));
    p->zs2prod = (cplx *)calloc(nom * njp * nvp * r->in.netot, sizeof(cplx));
    if (r->prod) {
        free(r->prod->nobcprod); free(r->prod->transrgjac); free(r->prod->dtrans); free(r->prod->prodwf);
        free(r->prod->cvjprod); free(r->prod->zs2prod); free(r->prod);
    }
    r->prod = p;
    return 0;
}

int mw3ref_get_product(const mw3ref *r, double *zs2prod, double *cvjprod)
{
    const prodproj *p = r->prod;
    if (!p) return 1;
    size_t n = (size_t)(p->om1 - p->om0 + 1) * (p->jp1 - p->jp0 + 1) * (p->vp1 - p->vp0 + 1);
    if (zs2prod) memcpy(zs2prod, p->zs2prod, sizeof(cplx) * n * r->in.netot);
    if (cvjprod) memcpy(cvjprod, p->cvjprod, sizeof(double) * n);
    return 0;
}

int mw3ref_start(mw3ref *r, const double *psi0)
{
    if (r->in.iphoto >= 1) {        /* check's rpaq0 (main_madwave3.f:444-455) */
        if (!r->psi0) r->psi0 = (double *)malloc(sizeof(double) * r->ntot);
        memcpy(r->psi0, psi0, sizeof(double) * r->ntot);
    }
    int64_t n = r->ntot;
    memcpy(r->psi_km1, psi0, sizeof(double) * n);
    memcpy(r->psi_k, psi0, sizeof(double) * n);
    difs(r, r->psi_k, r->hpsi);
    for (int64_t i = 0; i < n; i++)
        r->psi_k[i] = (r->hpsi[i] - r->in.emindlt * r->psi_km1[i]) / r->in.delta2;
    r->it = 1;
    return 0;
}

int mw3ref_run(mw3ref *r, int nit, double *norms)
{
    const mw3ref_in *in = &r->in;
    int n2 = r->n2, na = r->na, nc = r->nc;
    for (int s = 0; s < nit; s++) {
        int64_t it = r->it + 1;
        difs(r, r->psi_k, r->hpsi);
        for (int ia = 0; ia < na; ia++) {
            int iang = r->aorder[ia];
            int np = in->npunreal[iang - 1];
            for (int b = 0; b < nc; b++) {
                int64_t i0 = r->offs[(size_t)(iang - 1) * nc + b];
                for (int ir = 0; ir < np; ir++) {
                    int ir1 = in->indr1[(size_t)(iang - 1) * in->npuntot + ir];
                    int ir2 = in->indr2[(size_t)(iang - 1) * in->npuntot + ir];
                    int64_t i = i0 + ir;
                    double fabs_ = r->absfr1[ir1 - 1] * r->absfr2[ir2 - 1];
                    double rhnorm = (r->hpsi[i] - in->emindlt * r->psi_k[i]) / in->delta2;
                    double xxx = (2.0 * rhnorm - fabs_ * r->psi_km1[i]) * fabs_;
                    r->psi_km1[i] = r->psi_k[i];
                    r->psi_k[i] = xxx;
                }
            }
        }
        (void)n2;
        mw3ref_coefecheby(r, it, (double *)r->zck);
        if (r->n1 > 1) totalflux_k(r, it);
        if (r->n2 > 1) cvjflux_k(r, it);
        if (r->prod && r->n1 > 1 && r->n2 > 1) {
            prodpaq(r);
            prodcvj(r);
        }
        if (norms) {
            double x = 0.0;
            for (int64_t i = 0; i < r->ntot; i++) x = x + r->psi_k[i] * r->psi_k[i];
            norms[s] = x;
        }
        if (r->psi0) {
            double x = 0.0;
            for (int64_t i = 0; i < r->ntot; i++) x = x + r->psi0[i] * r->psi_k[i];
            r->autocor = x;
        }
        if (in->nofe > 0) fune(r, it);
        r->it = it;
    }
    return 0;
}

double mw3ref_autocorrelation(const mw3ref *r) { return r->autocor; }

int mw3ref_get_state(const mw3ref *r, double *psi_km1, double *psi_k, int64_t *it)
{
    if (psi_km1) memcpy(psi_km1, r->psi_km1, sizeof(double) * r->ntot);
    if (psi_k) memcpy(psi_k, r->psi_k, sizeof(double) * r->ntot);
    if (it) *it = r->it;
    return 0;
}

int mw3ref_set_state(mw3ref *r, const double *psi_km1, const double *psi_k, int64_t it)
{
    memcpy(r->psi_km1, psi_km1, sizeof(double) * r->ntot);
    memcpy(r->psi_k, psi_k, sizeof(double) * r->ntot);
    r->it = it;
    return 0;
}

/* totalflux (mod_flux_01y2.f:778-816) */
int mw3ref_totalflux(mw3ref *r, double *s2prodtot, double *s2prodelec)
{
    const mw3ref_in *in = &r->in;
    int netot = in->netot, ne = in->nelec;
    for (int ie = 0; ie < netot; ie++) {
        double s = 0.0;
        double *se = (double *)calloc(ne, sizeof(double));
        for (int f = 0; f < r->nflux; f++) {
            cplx a = r->zcr[(size_t)f * netot + ie], b = r->zcdr[(size_t)f * netot + ie];
            double im = a.re * b.im + (-a.im) * b.re;
            s = s + im;
            int ielec = in->nelebas[r->fl_can[f]];
            se[ielec - 1] = se[ielec - 1] + im;
        }
        s2prodtot[ie] = s * r->reacfct[ie] / in->ah1;
        if (s2prodelec)
            for (int e = 0; e < ne; e++) s2prodelec[(size_t)e * netot + ie] = se[e] * r->reacfct[ie] / in->ah1;
        free(se);
    }
    return 0;
}

int mw3ref_nflux(const mw3ref *r) { return r->nflux; }

int mw3ref_get_flux(const mw3ref *r, double *zcr, double *zcdr)
{
    size_t n = (size_t)r->nflux * r->in.netot;
    if (zcr) memcpy(zcr, r->zcr, sizeof(cplx) * n);
    if (zcdr) memcpy(zcdr, r->zcdr, sizeof(cplx) * n);
    return 0;
}

int mw3ref_get_s2(const mw3ref *r, double *zs2, double *cvj)
{
    size_t n = (size_t)r->nc * r->nj * r->nv;
    if (zs2) memcpy(zs2, r->zs2, sizeof(cplx) * n * r->in.netot);
    if (cvj) memcpy(cvj, r->cvj, sizeof(double) * n);
    return 0;
}

int mw3ref_get_zfe(const mw3ref *r, double *zfe)
{
    if (!r->zfe) return -1;
    memcpy(zfe, r->zfe, sizeof(cplx) * (size_t)r->in.nofe * r->ntot);
    return 0;
}

int mw3ref_tables(const mw3ref *r, int32_t *nopr1, double *p2r1, double *p2r2,
                  double *absfr1, double *absfr2, int32_t *irabs)
{
    int na = r->na;
    if (nopr1) for (int a = 0; a < na; a++) nopr1[a] = r->nopr1[a];
    if (p2r1) memcpy(p2r1, r->p2r1, sizeof(double) * (size_t)na * r->n1);
    if (p2r2) memcpy(p2r2, r->p2r2, sizeof(double) * (size_t)na * r->n2);
    if (absfr1) memcpy(absfr1, r->absfr1, sizeof(double) * r->n1);
    if (absfr2) memcpy(absfr2, r->absfr2, sizeof(double) * r->n2);
    if (irabs) { irabs[0] = r->ir1abs; irabs[1] = r->ir2abs; }
    return 0;
}

int mw3ref_flux_tables(const mw3ref *r, double *etot, double *reacfct, double *apaqini,
                       double *zar1flux, int32_t *ir4flux)
{
    int netot = r->in.netot;
    if (etot) memcpy(etot, r->etot, sizeof(double) * netot);
    if (reacfct) memcpy(reacfct, r->reacfct, sizeof(double) * netot);
    if (apaqini) memcpy(apaqini, r->apaqini, sizeof(double) * netot);
    if (zar1flux) memcpy(zar1flux, r->zar1flux, sizeof(cplx) * r->n1);
    if (ir4flux) *ir4flux = r->ir4flux;
    return 0;
}

int mw3ref_s2factor(const mw3ref *r, double *s2factor)
{
    memcpy(s2factor, r->s2factor, sizeof(double) * (size_t)r->in.nelec * r->nj * r->nv * r->in.netot);
    return 0;
}

int mw3ref_xj2(const mw3ref *r, double *xj2)
{
    memcpy(xj2, r->xj2, sizeof(double) * (size_t)r->nc * r->na * r->na * r->n1);
    return 0;
}

int mw3ref_xl2p(const mw3ref *r, double *xl2p)
{
    memcpy(xl2p, r->xl2p, sizeof(double) * 3 * (size_t)r->nc * r->na * r->na * r->n2);
    return 0;
}

/* ---------------------------------------------------------------------- */
/* stand-alone restatements for the known-answer tests                    */
/* ---------------------------------------------------------------------- */
int mw3ref_noptfft(int nin, int ntot) { return noptfft(nin, ntot); }

void mw3ref_sinmom_p2(double box, int npun, double xmred, double hbr, double *p2r)
{
    sinmom(box, npun, npun, xmred, hbr, NULL, p2r);
}

/* one direction of ini_absorcion (mod_absorcion_01y2.f:72-100) */
void mw3ref_absorption(int npun, double rmis, double ah, double absr, double absalp, int nexpo,
                       int ninterv, double *f, int32_t *irabs)
{
    *irabs = npun;
    for (int ir = 1; ir <= npun; ir++) {
        double r = (double)(ir - 1) * ah + rmis;
        double v = 1.0;
        if (r >= absr) {
            if (ir < *irabs) *irabs = ir;
            double delta = (r - absr) / (double)ninterv;
            v = exp(-(absalp * powi(delta, nexpo)));
        }
        f[ir - 1] = v;
    }
}

/* Smatini_col (mod_flux_01y2.f:392-524), energy part */
double mw3ref_smatini_col(int netot, double ekinmin, double ekinmax, double rmis2, double rfin2,
                          double rcolini, double xk0, double alpha0, double factor0, double xmasa0,
                          double xm1reac, int il0, double hbr, double *etot, double *apaqini,
                          double *reacfct)
{
    double estep = (ekinmax - ekinmin) / (double)(netot - 1);
    const int npunt = 1000;
    double rg[1000];
    double ahgauss = (rfin2 - rmis2) / (double)(npunt - 1);
    for (int ir2 = 1; ir2 <= npunt; ir2++) {
        double r2 = rmis2 + (double)(ir2 - 1) * ahgauss;
        double g = cos((r2 - rcolini) * xk0) * sqrt(2.0);
        rg[ir2 - 1] = g * factor0 * exp(-(r2 - rcolini) * (r2 - rcolini) / alpha0 / alpha0) / sqrt(2.0);
    }
    double pepe = (double)(il0 * (il0 + 1));
    double rr = rcolini + 1.0;
    double erot = hbr * hbr * pepe * 0.5 / (rr * rr * xmasa0);
    double xnorm = 0.0;
    for (int ie = 0; ie < netot; ie++) {
        double e = ekinmin + (double)ie * estep;
        double paqini = 0.0, pini = 0.0;
        if (e > 0.0 && e > erot) {
            pini = sqrt(e * xmasa0 * 2.0 / hbr / hbr);
            double zr = 0.0, zi = 0.0;
            for (int ir2 = 1; ir2 <= npunt; ir2++) {
                double rx = rmis2 + (double)(ir2 - 1) * ahgauss;
                double fb, gb;
                mw3ref_riccati(il0, rx * pini, &fb, &gb);
                if (fabs(fb) > 1e-20) { zr += rg[ir2 - 1] * (-gb); zi += rg[ir2 - 1] * fb; }
            }
            zr = zr * ahgauss / 2.0 / MW3_PI;
            zi = zi * ahgauss / 2.0 / MW3_PI;
            paqini = zr * zr + zi * zi;
        }
        if (etot) etot[ie] = e;
        if (apaqini) apaqini[ie] = paqini;
        xnorm = xnorm + paqini;
        if (reacfct)
            reacfct[ie] = (paqini < 1e-10) ? 0.0 : hbr * hbr * pini / paqini / xmasa0 / xm1reac / 4.0 / MW3_PI / MW3_PI;
    }
    return xnorm * estep;
}
