/*
 * mw3ref -- CPU oracle for the madwave3 Chebyshev hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a loop-by-loop restatement, in plain C
 * and FP64, of the reference's H.psi application and Chebyshev loop; it is
 * the checker the GPU path is compared against and the CPU baseline that
 * bench.py times.  Nothing in the product (madwave3_gb300/, libmw3gpu.so)
 * links or calls it.
 *
 * Restated reference routines (file:line inside octavioroncero/madwave3):
 *   Tradial            SRC/mod_Hphi_01y2.f:487-620 (noptFFT liboctdyn.f:1033-1117,
 *                      sinmom liboctdyn.f:1004-1031, fftmom liboctdyn.f:1119-1152)
 *   angkinj2           SRC/mod_Hphi_01y2.f:166-311   -> explicit xj2
 *   angkinj2 (eCoriolis) SRC/mod_Hphi_eCoriolis_01y2.f:186-324 -> channel-pair xj2,
 *                      applied as in its difs :901-911 (mw3ref_set_ecoriolis)
 *   bfgridl2mat        SRC/mod_Hphi_01y2.f:315-484   -> explicit xl2p (l2mat liboctdyn.f:1944-1990)
 *   difs               SRC/mod_Hphi_01y2.f:623-943   (T, V and j^2+l^2 parts, single process)
 *   ini_absorcion      SRC/mod_absorcion_01y2.f:28-107
 *   ini_flux           SRC/mod_flux_01y2.f:54-334
 *   Smatini_col        SRC/mod_flux_01y2.f:392-524
 *   totalflux_k        SRC/mod_flux_01y2.f:585-660
 *   Cvjflux_k          SRC/mod_flux_01y2.f:663-775
 *   totalflux          SRC/mod_flux_01y2.f:778-816
 *   funE               SRC/mod_PsiE_01y2.f:92-123
 *   CoefEcheby         SRC/main_madwave3.f:462-490
 *   check              SRC/main_madwave3.f:414-458
 *   first step/update  SRC/main_madwave3.f:238-250, 324-339
 *
 * Third-party arithmetic: FFTW3's RODFT00 (DST-I), whose documented
 * definition Y_k = 2 sum_j X_j sin(pi (j+1)(k+1)/(n+1)) is restated both as
 * the direct sum and through a complex FFT of the odd extension.
 *
 * All arrays are C row-major with the slowest index first; see mw3ref_in.
 */
#ifndef MW3REF_H
#define MW3REF_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    /* grid (mod_gridYpara) and pot0 */
    int32_t npun1, npun2, nangu, nangu2, nelec, npun1min;
    double rmis1, rfin1, ah1, rmis2, rfin2, ah2;
    double hbr, xm1red, xm2red, xm1reac, xm2reac;
    double vcutmax, radcutmax, rotcutmax;
    double emindlt, delta2;
    int32_t proj_j2_up;
    /* compressed grid (pot2): npunreal[nangu], indr1/indr2[nangu][npuntot] (1-based),
       vvv[je][ie][iang][ir]  = VVV(ir,iang,ie,je) */
    int32_t npuntot;
    const int32_t *npunreal, *indr1, *indr2;
    const double *vvv;
    /* basis for one partial wave */
    int32_t Jtot, iparity, inc, j0, iommin, iommax;
    int32_t ncan;
    const int32_t *iombas, *nelebas, *nojbas, *j00, *jbas;   /* jbas[ncan][nangu] */
    const int32_t *iomdiat, *iomatom;                         /* [nelec] */
    const double *sigdiat, *sigatom;                          /* [nelec] */
    const double *djmmp;            /* [Jtot+1][nelec][nangu2+1][nangu] */
    /* absorption namelist */
    double absr1, absalp1, absr2, absalp2;
    int32_t n1expo, ninterv1, n2expo, ninterv2;
    /* flux namelist and reference state */
    double r1flux_ang, ekinmin, ekinmax;   /* ekin* in zots */
    int32_t netot, kminelastic, iphoto, iprod;
    int32_t nvini, nvmax, jini, jmax, nvref, jref, iomref, ielecref;
    const int32_t *nobc;            /* [nelec][jmax-jini+1] */
    const double *ediat;            /* [nelec][nj][nv]  */
    const double *fd;               /* [nelec][nj][nv][npun1] */
    /* collision packet parameters (mod_colini) */
    double rcolini, alpha0, xk0, factor0, xmasa0;
    int32_t il0;
    /* PsiE */
    int32_t nofe;
    const double *efe;              /* [nofe] zots */
} mw3ref_in;

typedef struct mw3ref mw3ref;

mw3ref *mw3ref_create(const mw3ref_in *in, char *err, int errlen);
void mw3ref_destroy(mw3ref *r);
int64_t mw3ref_ntot(const mw3ref *r);
void mw3ref_set_threads(mw3ref *r, int nthreads);
void mw3ref_set_dst_mode(mw3ref *r, int mode);      /* 0 = FFT, 1 = direct sum */
void mw3ref_set_flux_gate(mw3ref *r, int on);       /* totalflux_k's E > V(flux point) test, default on */
void mw3ref_set_ecoriolis(mw3ref *r, int on);      /* the electronic Coriolis H (mod_Hphi_eCoriolis_01y2.f), default off */
double mw3ref_autocorrelation(const mw3ref *r);     /* iphoto >= 1: <psi0|psi_k> of the last iteration */

/* difs: hpsi = H psi (flat reference layout) */
int mw3ref_hphi(mw3ref *r, const double *psi, double *hpsi);
/* main_madwave3.f:238-250: psi_{k-1}=psi0, psi_k=(H psi0 - emindlt psi0)/delta2, it=1 */
int mw3ref_start(mw3ref *r, const double *psi0);
/* n iterations of main_madwave3.f:324-352 (difs, update, CoefEcheby, totalflux_k,
   Cvjflux_k, check, funE); norms[i] = ||psi_k||^2 after iteration i (may be NULL) */
int mw3ref_run(mw3ref *r, int n, double *norms);
int mw3ref_get_state(const mw3ref *r, double *psi_km1, double *psi_k, int64_t *it);
int mw3ref_set_state(mw3ref *r, const double *psi_km1, const double *psi_k, int64_t it);
/* totalflux: S2prodtot[netot], S2prodelec[nelec][netot] (may be NULL) */
int mw3ref_totalflux(mw3ref *r, double *s2prodtot, double *s2prodelec);
/* accumulators: zcr/zcdr [nflux][netot] complex (re,im), zs2 [ncan][nj][nv][netot] complex,
   cvj [ncan][nj][nv] (last iteration) */
int mw3ref_nflux(const mw3ref *r);
int mw3ref_get_flux(const mw3ref *r, double *zcr, double *zcdr);
int mw3ref_get_s2(const mw3ref *r, double *zs2, double *cvj);
int mw3ref_get_zfe(const mw3ref *r, double *zfe);     /* [nofe][ntot] complex */
/* set-up tables, for tests: ck[netot] complex for iteration k */
int mw3ref_coefecheby(const mw3ref *r, int64_t k, double *ck);
int mw3ref_tables(const mw3ref *r, int32_t *nopr1, double *p2r1, double *p2r2,
                  double *absfr1, double *absfr2, int32_t *ir1abs_ir2abs);
int mw3ref_flux_tables(const mw3ref *r, double *etot, double *reacfct, double *apaqini,
                       double *zar1flux, int32_t *ir4flux);
int mw3ref_s2factor(const mw3ref *r, double *s2factor);  /* [nelec][nj][nv][netot] */
/* product-state projection (iprod = 2, prodpaq/prodcvj): the tables ini_transcoor
   builds, in the C order of the Fortran arrays: transrgjac[ntot],
   dtrans[ncan][nom][nang][n2p], prodwf[nom][njp][nvp][nelec][nang][n2p],
   nobcprod[njp]; results zs2prod[nom][njp][nvp][netot] complex, cvjprod[nom][njp][nvp] */
int mw3ref_set_product(mw3ref *r, int n2prod0, int n2prod1, int nangproj0, int nangproj1, int iomminprod,
                       int iommaxprod, int jiniprod, int jmaxprod, int nviniprod, int nvmaxprod,
                       const int32_t *nobcprod, const double *transrgjac, const double *dtrans,
                       const double *prodwf);
int mw3ref_get_product(const mw3ref *r, double *zs2prod, double *cvjprod);
int mw3ref_xj2(const mw3ref *r, double *xj2);    /* [ncan][nangu(jang)][nangu(iang)][npun1] */
int mw3ref_xl2p(const mw3ref *r, double *xl2p);  /* [3][ncan][nangu][nangu][npun2] */
/* Stand-alone restatements used by the known-answer tests against the
   reference's golden log (EXAMPLES/HD+H_collision/J000-check/sal.000). */
int mw3ref_noptfft(int nin, int ntot);
void mw3ref_sinmom_p2(double box, int npun, double xmred, double hbr, double *p2r);
void mw3ref_absorption(int npun, double rmis, double ah, double absr, double absalp, int nexpo,
                       int ninterv, double *f, int32_t *irabs);
/* Smatini_col energy grid and packet projection; returns sum(apaqini)*estep,
   the "Norm ini. wvp in energy" line of the log */
double mw3ref_smatini_col(int netot, double ekinmin, double ekinmax, double rmis2, double rfin2,
                          double rcolini, double xk0, double alpha0, double factor0, double xmasa0,
                          double xm1reac, int il0, double hbr, double *etot, double *apaqini,
                          double *reacfct);
/* DST-I of one line (RODFT00), exposed for the known-answer tests */
void mw3ref_dst1(int n, const double *x, double *y, int mode);
void mw3ref_riccati(int l, double x, double *f, double *g);

#ifdef __cplusplus
}
#endif
#endif
