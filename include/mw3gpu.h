/*
 * mw3gpu.h -- C-ABI of the GB300 Chebyshev wave-packet propagator.
 *
 * Drop-in for the H.psi application and the Chebyshev loop that madwave3's
 * main program drives.  In the reference these are argument-less Fortran
 * module routines sharing module state; here they are functions on an opaque
 * context.  Every entry point returns 0 (MW3_OK) on success, a positive
 * MW3_ERR_* code otherwise; mw3_last_error() gives the message.  The host
 * (Fortran through iso_c_binding, or C/C++/Python) owns every input array and
 * may free it after the call that takes it: the library copies what it needs.
 *
 * Array conventions: all arrays are C row-major, slowest index first.  A
 * Fortran array A(n1,n2,n3) passes unchanged as C A[n3][n2][n1].  Grid indices
 * stored in arrays (indr1, indr2, jbas) keep the reference's 1-based values.
 * State vectors use the reference's flat layout for one process
 * (indtotproc, SRC/mod_pot_01y2.f:435-455): angles in the order
 * nangu, nangu-1, ..., 1, then Omega/electronic block, then stored point.
 *
 * Threading: one host thread per context; calls on one context must not
 * overlap.  All device work of a context runs on its own CUDA stream.
 */
#ifndef MW3GPU_H
#define MW3GPU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MW3_OK 0
#define MW3_ERR_ARG 1          /* invalid argument or inconsistent sizes */
#define MW3_ERR_CUDA 2         /* CUDA runtime error */
#define MW3_ERR_UNSUPPORTED 3  /* input the library does not implement */
#define MW3_ERR_STATE 4        /* call out of order */
#define MW3_ERR_NOMEM 5        /* device allocation failed */
#define MW3_ERR_NUMERIC 6      /* non-finite values detected in the state */

#define MW3_PREC_FP64 0        /* FP64 throughout (the reference's arithmetic) */
#define MW3_PREC_MIXED 1       /* FP32 transforms, FP64 recursion and accumulators */

typedef struct mw3_ctx mw3_ctx;

/* Grid, masses, cut-offs and the compressed potential grid shared by every
 * partial wave of a context.  Replaces what mod_gridYpara_01y2 and
 * mod_pot_01y2 (pot0, pot2) hold for mod_Hphi_01y2
 * (SRC/mod_gridYpara_01y2.f:38-77, SRC/mod_pot_01y2.f:16-48). */
typedef struct {
    int32_t npun1, npun2, nangu, nelec;   /* r1 points, r2 points, angles, electronic states */
    int32_t npun1min;                     /* minimum DST length in r1 (&inputgridbase) */
    int32_t npuntot;                      /* max(npunreal): leading dimension of indr1/indr2/vvv */
    double rmis1, rfin1, rmis2, rfin2;    /* radial grid ends, angstrom */
    double hbr;                           /* hbar in zot units (mod_gridYpara_01y2.f:21) */
    double xm1red, xm2red;                /* reduced masses, amu */
    double radcutmax, rotcutmax;          /* kinetic cut-offs, zots */
    double emindlt, delta2;               /* Chebyshev centre and half width, zots (pot2 :502-505) */
    int32_t precision;                    /* MW3_PREC_FP64 or MW3_PREC_MIXED */
} mw3_grid;

/* One partial wave J: its basis and the namelist values of the modules the
 * library replaces (mod_absorcion_01y2, mod_flux_01y2, mod_colini's packet
 * parameters for Smatini_col). */
typedef struct {
    int32_t Jtot, iparity, inc, j0, iommin, iommax;
    int32_t ncan;                         /* number of (electronic state, Omega) blocks */
    const int32_t *iombas, *nelebas;      /* [ncan]; nelebas 1-based */
    const int32_t *nojbas, *j00;          /* [ncan] */
    const int32_t *jbas;                  /* [ncan][nangu] */
    const int32_t *iomdiat, *iomatom;     /* [nelec] */
    const double *sigdiat, *sigatom;      /* [nelec] */
    int32_t nangu2;                       /* nangu*inc */
    const double *djmmp;                  /* Djmmp(nangu,0:nangu2,nelec,0:Jtot) = [Jtot+1][nelec][nangu2+1][nangu] */
    int32_t proj_j2_up;                   /* must be 0 */
    /* &inputabsorcion */
    double absr1, absalp1, absr2, absalp2;
    int32_t n1expo, ninterv1, n2expo, ninterv2;
    /* &inputflux, reference state and process */
    double r1flux_ang, ekinmin, ekinmax;  /* ekin in zots */
    int32_t netot, kminelastic, iphoto, iprod;
    int32_t nvini, nvmax, jini, jmax, nvref, jref, iomref, ielecref;
    const int32_t *nobc;                  /* noBCstates(jini:jmax,nelec) = [nelec][nj] */
    const double *ediat;                  /* ediat(nvini:nvmax,jini:jmax,nelec) = [nelec][nj][nv] */
    const double *fd;                     /* fd(npun1,nvini:nvmax,jini:jmax,nelec) = [nelec][nj][nv][npun1] */
    double xm1reac, xm2reac;
    double rcolini, alpha0, xk0, factor0, xmasa0;   /* mod_colini_01y2 */
    int32_t il0;
    int32_t nofe;                         /* &inputPsiE: number of energies, 0 = off */
    const double *efe;                    /* [nofe] zots */
} mw3_wave;

/* Create a context on the current CUDA device.  npunreal[nangu],
 * indr1/indr2[nangu][npuntot], vvv[nelec][nelec][nangu][npuntot] with
 * vvv[je][ie][iang][ir] = VVV(ir,iang,ie,je).
 * Replaces pot2's device-side state (SRC/mod_pot_01y2.f:344-533). */
int mw3_create(mw3_ctx **ctx, const mw3_grid *grid, const int32_t *npunreal,
               const int32_t *indr1, const int32_t *indr2, const double *vvv);

/* Add one partial wave; builds the kinetic, absorption and flux tables
 * (set_vectors_Hphi SRC/mod_Hphi_01y2.f:38-163, ini_absorcion
 * SRC/mod_absorcion_01y2.f:28-107, ini_flux/Smatini_col
 * SRC/mod_flux_01y2.f:54-524, input_PsiE SRC/mod_PsiE_01y2.f:19-88).
 * *wave_id receives its index (0, 1, ...). */
int mw3_add_wave(mw3_ctx *ctx, const mw3_wave *wave, int32_t *wave_id);

/* Number of doubles in a wave's state vector (ntotproc, one process). */
int mw3_wave_size(mw3_ctx *ctx, int32_t wave_id, int64_t *ntot);

/* difs: hpsi = H psi for one wave, host arrays in and out
 * (SRC/mod_Hphi_01y2.f:623-943).  Leaves the propagation state unchanged. */
int mw3_hphi(mw3_ctx *ctx, int32_t wave_id, const double *psi, double *hpsi);

/* Fresh start of every wave from its initial packet psi0 (host array):
 * psi_{k-1} = psi0, psi_k = (H psi0 - emindlt psi0)/delta2, k = 1
 * (SRC/main_madwave3.f:238-250).  psi0s[w] points at wave w's vector. */
int mw3_start(mw3_ctx *ctx, const double *const *psi0s);

/* Restart from stored vectors (cont##.paq, SRC/main_madwave3.f:253-260). */
int mw3_upload_state(mw3_ctx *ctx, int32_t wave_id, const double *psi_km1,
                     const double *psi_k, int64_t it);

/* n Chebyshev iterations of every wave, device resident: difs, the damped
 * three-term update, CoefEcheby, totalflux_k, Cvjflux_k, check and funE
 * (SRC/main_madwave3.f:324-352). */
int mw3_run(mw3_ctx *ctx, int64_t n_iter);

/* Wait for queued work; reports a deferred CUDA error. */
int mw3_sync(mw3_ctx *ctx);

int mw3_download_state(mw3_ctx *ctx, int32_t wave_id, double *psi_km1, double *psi_k,
                       int64_t *it);

/* mw3_upload_state / mw3_download_state for every wave at once: the host arrays
 * hold the waves' vectors back to back in wave order (wave w starts after the
 * ntot of waves 0..w-1), moved with one copy each way for the whole context and
 * one synchronisation per call.  Once the context holds a state, psi_km1 may
 * be NULL: the device keeps its current psi_{k-1} and only psi_k is replaced
 * (a host loop that reads psi_k back every iteration and hands it in again). */
int mw3_upload_state_all(mw3_ctx *ctx, const double *psi_km1, const double *psi_k, int64_t it);
int mw3_download_state_all(mw3_ctx *ctx, double *psi_km1, double *psi_k, int64_t *it);

/* ||psi_k||^2 after each iteration since the last mw3_start/upload
 * (check, SRC/main_madwave3.f:431-442): norms[0..*n-1]; *n in: capacity,
 * out: number written. */
int mw3_norms(mw3_ctx *ctx, int32_t wave_id, double *norms, int64_t *n);

/* totalflux (SRC/mod_flux_01y2.f:778-816): P(E) and per-state split.
 * s2prodtot[netot], s2prodelec[nelec][netot] (may be NULL). */
int mw3_totalflux(mw3_ctx *ctx, int32_t wave_id, double *s2prodtot, double *s2prodelec);

/* check's autocorrelation for photodissociation waves (iphoto >= 1,
 * SRC/main_madwave3.f:444-455, written to the auto.* file the spectra program
 * reads): <psi0|psi_k> after each iteration since the last mw3_start, with
 * psi0 the packet mw3_start received; same slots as mw3_norms. */
int mw3_autocorrelation(mw3_ctx *ctx, int32_t wave_id, double *autos, int64_t *n);

/* Raw accumulators, complex as (re,im) pairs: zcr/zcdr [nflux][netot],
 * zs2 [ncan][nj][nv][netot], cvj [ncan][nj][nv] of the last iteration,
 * zfe [nofe][ntot].  Any pointer may be NULL. */
int mw3_flux_count(mw3_ctx *ctx, int32_t wave_id, int32_t *nflux);
int mw3_download_accumulators(mw3_ctx *ctx, int32_t wave_id, double *zcr, double *zcdr,
                              double *zs2, double *cvj, double *zfe);

/* Set-up tables for inspection: nopr1[nangu], reacfct[netot], S2factor
 * [nelec][nj][nv][netot], etot[netot], absfr1[npun1], absfr2[npun2]. */
/* Continuation: the accumulators a restart reads back from cont##.S2
 * (SRC/mod_flux_01y2.f:296-320; written by wvpcont, SRC/main_madwave3.f:519-525),
 * same layouts as mw3_download_accumulators (any pointer may be NULL).  Call
 * after the state (mw3_upload_state / mw3_upload_state_all): every wave's
 * pending ring samples are added first, then this wave's accumulators are
 * replaced. */
int mw3_upload_accumulators(mw3_ctx *ctx, int32_t wave_id, const double *zcr, const double *zcdr,
                            const double *zs2);
int mw3_tables(mw3_ctx *ctx, int32_t wave_id, int32_t *nopr1, double *etot, double *reacfct,
               double *s2factor, double *absfr1, double *absfr2);

/* Per-iteration Cvj and Cvjprod, the records the reference writes every
 * iteration to Cvj.NNNN / Cvjprod.NNNN (write(15) it, Cvj and write(16) it,
 * Cvjprod, SRC/main_madwave3.f:310-321, 354-364): mw3_cvj_history keeps them
 * on the device in a ring of `capacity` iterations (0 turns it off), filled by
 * every iteration of mw3_run since the last mw3_start / upload; the host
 * drains it once per ntimes block.  mw3_download_cvj_history returns the last
 * n recorded iterations, oldest first: cvj[n][ncan][nj][nv] (the wave's Cvj,
 * Fortran Cvj(nvini:nvmax,jini:jmax,ncan)) and, for a wave with a product
 * projection, cvjprod[n][nom][njp][nvp]; either may be NULL.  *it_last is the
 * iteration of the newest record. */
int mw3_cvj_history(mw3_ctx *ctx, int64_t capacity);
int mw3_download_cvj_history(mw3_ctx *ctx, int32_t wave_id, int64_t n, double *cvj, double *cvjprod,
                             int64_t *it_last);

/* totalflux_k's energy test (SRC/mod_flux_01y2.f:640): with on != 0 (the
 * default, as the shipped source) the flux through a point counts only at the
 * energies above its potential; with on = 0 every energy takes every flux
 * point, the earlier form of the routine with which the reference's shipped
 * H + HD run (EXAMPLES/HD+H_collision/J000-check) was made.  Call before the
 * context's device tables exist, else MW3_ERR_STATE. */
int mw3_set_flux_gate(mw3_ctx *ctx, int32_t wave_id, int32_t on);

/* The electronic Coriolis Hamiltonian of the reference's mad3renner build
 * (SRC/mod_Hphi_eCoriolis_01y2.f, linked in place of mod_Hphi_01y2.f): with
 * on != 0 the wave's H psi adds the j^2-type coupling between channels of
 * equal Omega and sigma whose diatomic Lambda (iomdiat) differ by one
 * (angkinj2 :226-285, difs :901-911); off (the default) is the plain difs.
 * Replaces linking the eCoriolis module: the same mw3_hphi / mw3_run calls
 * then apply it.  Call before the context's device tables exist, else
 * MW3_ERR_STATE. */
int mw3_set_ecoriolis(mw3_ctx *ctx, int32_t wave_id, int32_t on);

/* Path choices and the autotuner (no counterpart in the reference, whose
 * single CPU code path has none).  choice[4]:
 *   [0] radial DST form -- mixed: 0 fused split-FP16 tcgen05 chain, 1 fused
 *       3xTF32 chain, 2 three-kernel tensor-core DST, 3 CUDA-core FP32 DST;
 *       FP64: 0 folded dense DST-I, 1 Rader FFT along R (npun2 = 256);
 *   [1] FP32 rectangle stored [R][r1]: 0 no, 1 yes (where eligible);
 *   [2] mixed angular terms: 0 explicit kernels, 1 factorised tensor-core kernel;
 *   [3] R-column chunk of the explicit angular kernels: 8..64, a power of two;
 * -1 (0 for [3]) keeps the built-in rule, and a form the shape does not admit
 * falls back to the next one that it does.  Call before mw3_start. */
int mw3_set_choices(mw3_ctx *ctx, const int32_t *choice);
int mw3_get_choices(mw3_ctx *ctx, int32_t *choice);

#define MW3_TUNE_LAYOUT 1   /* rectangle layout, angular column chunk: results unchanged bit for bit */
#define MW3_TUNE_FORM 2     /* DST factorisation and angular form: results change at the rounding level */
/* Times `iterations` (rounded up to a multiple of 64) propagation iterations
 * of the context's waves from a synthetic state for every distinct path the
 * choices in `scope` allow, each after a warm-up that captures the iteration
 * graphs, and keeps the fastest: the context is left built with it and not
 * started, its choices in choice[4], its time per iteration in *ms_best
 * (either may be NULL).  Call after mw3_add_wave (and any mw3_set_*), before
 * mw3_start; the device tables are rebuilt once per candidate. */
int mw3_autotune(mw3_ctx *ctx, int32_t iterations, int32_t scope, int32_t *choice, double *ms_best);

/* apaqini[netot]: the energy distribution |<packet|E>|^2 of the initial
 * collision packet that Smatini_col computes (SRC/mod_flux_01y2.f:467-524) and
 * the reference keeps in mod_flux for its normalisations -- ini_transcoor's
 * S2prodfac (SRC/mod_coortrans01_02.f:121-145) among them. */
int mw3_packet_energy_norm(mw3_ctx *ctx, int32_t wave_id, double *apaqini);

/* Number of CUDA kernels this context has launched so far. */
int mw3_kernel_launches(mw3_ctx *ctx, int64_t *count);

/* Which kernels the context runs, valid once its device tables exist (after
 * mw3_start, mw3_upload_state or mw3_hphi): MW3_PATH_TC_DST when the radial
 * DSTs run on the tensor cores (with MW3_PATH_TC_DST_FUSED when as one fused
 * kernel, and MW3_PATH_DST_F16 when that kernel takes split-FP16 products
 * rather than 3xTF32), MW3_PATH_TC_ANG when the angular terms run as the
 * factorised tensor-core contraction (all mixed precision only).  No
 * reference counterpart: the reference has a single code path. */
#define MW3_PATH_TC_DST 1
#define MW3_PATH_TC_ANG 2
#define MW3_PATH_TC_DST_FUSED 4   /* the whole radial DST chain in one kernel per (block, angle) */
#define MW3_PATH_DST_F16 8        /* the fused chain as split-FP16 products (MW3_DST_TF32=1 selects 3xTF32) */
#define MW3_PATH_X_T 16           /* the FP32 rectangle stored [R][r1] (MW3_X_T=1; default [r1][R]) */
#define MW3_PATH_RADER 32         /* FP64: the DST along R by Rader's FFT (npun2 = 256) */
int mw3_path_flags(mw3_ctx *ctx, int32_t *flags);

/* The CUDA stream (cudaStream_t) all device work of the context runs on, for
 * callers that order their own work or timing events against it. */
int mw3_get_stream(mw3_ctx *ctx, void **stream);

/* Per-stage timing: while enabled, mw3_run records CUDA events around each
 * stage of every iteration.  mw3_stage_times waits for the stream and returns
 * the accumulated milliseconds of MW3_NSTAGES stages and the number of
 * iterations recorded, then clears the record. */
#define MW3_NSTAGES 7   /* R-DST (or the fused DST chain), r-DST pair, R-DST+gather, angular (j^2, or j^2+l^2 fused), l^2, update, accumulators */
int mw3_profile(mw3_ctx *ctx, int enable);
int mw3_stage_times(mw3_ctx *ctx, double *ms, int64_t *iterations);

/* H psi for one wave without allocating anything.
 *
 * No counterpart in the reference: it exists for callers that can allocate
 * GPU memory only while they start up, not inside their time loop -- for
 * example a host whose device memory is owned by another allocator that
 * holds the whole GPU, or a loop where the implicit device synchronisation
 * of cudaMalloc/cudaFree would stall every iteration.  psi and hpsi are
 * DEVICE pointers to the wave's state vector layout (mw3_wave_size doubles);
 * they must not overlap (MW3_ERR_ARG otherwise: psi is still read after
 * hpsi is first written).
 * The transform scratch lives in one file-scope device array of
 * MW3_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until
 * exit; waves whose scratch (two rectangles of ncan*nangu*npun1*npun2
 * elements, 8 bytes each in FP64, 4 in mixed) exceeds it are rejected with
 * MW3_ERR_UNSUPPORTED.  The context's device tables must already exist (any
 * earlier mw3_hphi, mw3_start or mw3_upload_state builds them).  The first
 * call on a device looks up the array's device address once (under a lock,
 * so threads may make it concurrently) and keeps it for the life of the
 * process, which assumes the device's primary context is not reset
 * (cudaDeviceReset) while the library is loaded; make that first call before
 * any stream capture.  All calls share the array, so calls that overlap on
 * the GPU (other threads or contexts on the same device) race.  Returns after
 * the result is in hpsi, with MW3_ERR_CUDA if a launch failed or a
 * tensor-core kernel gave up waiting for its MMAs. */
#define MW3_NOALLOC_SCRATCH_BYTES (64u << 20)
int mw3_hphi_noalloc(mw3_ctx *ctx, int32_t wave_id, const double *psi, double *hpsi);

/* Product-state projection (iprod = 2): prodpaq and prodcvj
 * (SRC/mod_coortrans01_02.f:694-825) every iteration of mw3_run, after the
 * Cvj projection.  The tables are the ones ini_transcoor builds
 * (SRC/mod_coortrans01_02.f:32-207, allocated at :90-97 and :255-260), passed
 * in Fortran order like every other table; ranges are inclusive, R and angle
 * indices 1-based.  Set before the context's device tables exist (before the
 * first mw3_hphi / mw3_start / mw3_upload_state), else MW3_ERR_STATE. */
typedef struct mw3_prodproj {
    int32_t n2prod0, n2prod1;             /* R range of the projection */
    int32_t nangproj0, nangproj1;         /* angle range */
    int32_t iomminprod, iommaxprod;       /* product Omega range */
    int32_t jiniprod, jmaxprod;           /* product j range */
    int32_t nviniprod, nvmaxprod;         /* product v range */
    const int32_t *nobcprod;              /* noBCprod(jiniprod:jmaxprod), each <= nvmaxprod */
    const double *transrgjac;             /* transRgjac on the wave's state vector (mw3_wave_size doubles) */
    const double *dtrans;                 /* dtrans(n2prod0:n2prod1,nangproj0:nangproj1,iomminprod:iommaxprod,ncan) */
    const double *prodwf;                 /* prodwf(n2prod0:n2prod1,nangproj0:nangproj1,nelec,
                                             nviniprod:nvmaxprod,jiniprod:jmaxprod,iomminprod:iommaxprod) */
} mw3_prodproj;
int mw3_set_product_projection(mw3_ctx *ctx, int32_t wave_id, const mw3_prodproj *proj);

/* zS2prod(netot,nviniprod:nvmaxprod,jiniprod:jmaxprod,iomminprod:iommaxprod)
 * complex as (re,im) pairs, and the last iteration's Cvjprod(v,j,Omega)
 * (either may be NULL). */
int mw3_download_product(mw3_ctx *ctx, int32_t wave_id, double *zs2prod, double *cvjprod);
/* zS2prod of a restart (cont##.S2prod, SRC/mod_coortrans01_02.f:183-197). */
int mw3_upload_product(mw3_ctx *ctx, int32_t wave_id, const double *zs2prod);

const char *mw3_last_error(const mw3_ctx *ctx);
int mw3_destroy(mw3_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif
