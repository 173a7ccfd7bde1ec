// Internal declarations of libmw3gpu: context layout, device tables and the
// kernel launchers shared by mw3_api.cu, mw3_setup.cu and mw3_kernels.cu.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <cstdlib>

#include <string>
#include <vector>

#include "../../include/mw3gpu.h"

namespace mw3 {

// ---------------------------------------------------------------------------
// host-side tables of one partial wave (what set_vectors_Hphi, ini_absorcion,
// ini_flux/Smatini_col and input_PsiE leave in module state)
// ---------------------------------------------------------------------------
struct WaveTables {
    // scalars copied from mw3_wave
    int Jtot, iparity, inc, j0, iommin, iommax, ncan, nangu2, proj_j2_up;
    double absr1, absalp1, absr2, absalp2;
    int n1expo, ninterv1, n2expo, ninterv2;
    double r1flux_ang, ekinmin, ekinmax;
    int netot, kminelastic, iphoto, iprod;
    int nvini, nvmax, jini, jmax, nvref, jref, iomref, ielecref;
    double xm1reac, xm2reac, rcolini, alpha0, xk0, factor0, xmasa0;
    int il0, nofe;
    std::vector<int> iombas, nelebas, nojbas, j00, jbas;   // jbas [ncan][nangu]
    std::vector<int> iomdiat, iomatom;
    std::vector<double> sigdiat, sigatom;
    std::vector<double> djmmp;                              // [Jtot+1][nelec][nangu2+1][nangu]
    std::vector<int> nobc;
    std::vector<double> ediat, fd, efe;
    int nj = 0, nv = 0;

    // layout
    int64_t ntot = 0;            // points of this wave
    int64_t flat0 = 0;           // start in the context-wide flat arrays
    int g0 = 0;                  // first context-wide block
    std::vector<int64_t> offs;   // [nangu][ncan] flat start relative to flat0

    // Tradial (mod_Hphi_01y2.f:487-620)
    std::vector<int> nopr1;                 // [nangu]
    std::vector<double> p2r1, p2r2;         // [nangu][npun1], [nangu][npun2]
    // angkinj2 scalar part: yyy(ir1, k) for the block's j list, [ncan][npun1][nangu]
    std::vector<double> yj2;
    // bfgridl2mat scalar part: xl2mat for (ielec, j, ir2, iom, jom)
    //   l2tab[((ielec*nj2 + jidx)*npun2 + ir2)*nom*nom + (iom-iommin)*nom + (jom-iommin)]
    int nj2 = 0, nom = 0;
    std::vector<double> l2tab;
    std::vector<char> l2used;               // [ielec][jidx][iom][jom] combination present
    // ini_absorcion
    std::vector<double> absfr1, absfr2;
    int ir1abs = 0, ir2abs = 0;
    // ini_flux
    int ir4flux = 0;
    std::vector<double> zar1flux;           // [npun1][2]
    std::vector<int> ir1flux;               // [nangu]
    int nflux = 0;
    std::vector<int64_t> fl_idx;            // flat index (wave-relative) of each flux point
    std::vector<int> fl_block;              // block of each flux point
    std::vector<double> potiflux;
    bool flux_gate = true;                  // totalflux_k's E > V(flux point) test
    bool ecor = false;                      // electronic Coriolis H (mod_Hphi_eCoriolis_01y2.f)
    std::vector<int> fl_dptr;               // CSR over flux points of the r1-derivative terms
    std::vector<int64_t> fl_didx;           // wave-relative flat index of each term
    std::vector<int> fl_dir1;               // ir1 (0-based) of each term
    // Smatini_col
    std::vector<double> etot, reacfct, apaqini, s2factor;
    int icanref = -1;
    // Cvjflux_k
    std::vector<int> r2abs_map;             // [nangu][npun1] local point index at ir2abs, or -1
};

// device pointers of one wave
// product-state projection of one wave (iprod = 2; prodpaq / prodcvj): the host's
// tables as given to mw3_set_product_projection
struct ProdTables {
    bool on = false;
    int n2p0 = 0, n2p1 = 0, a0 = 0, a1 = 0, om0 = 0, om1 = 0, jp0 = 0, jp1 = 0, vp0 = 0, vp1 = 0;
    std::vector<int> nobcprod;                   // [njp]
    std::vector<double> transrgjac;              // [ntot]
    std::vector<double> dtrans;                  // [ncan][nom][nang][n2p]
    std::vector<double> prodwf;                  // [nom][njp][nvp][nelec][nang][n2p]
};

// its device side: the points of every (block, angle, R) bin as a CSR list in
// the reference's summation order, the tables, and the results
struct ProdDev {
    int nbins = 0, nrow = 0;                     // bins = ncan nang n2p; rows = nom njp nvp
    int *bin_ptr = nullptr;                      // [nbins + 1]
    int64_t *bin_idx = nullptr;                  // context-wide flat index of each term
    double *bin_w = nullptr;                     // its transRgjac
    double *fun = nullptr;                       // funprod [ncan][nang][n2p]
    double *dtrans = nullptr, *prodwf = nullptr;
    int *nobcprod = nullptr, *blk_elec = nullptr;
    double *cvjprod = nullptr;                   // [nrow]
    double *cvjph = nullptr;                     // [hist_cap][nrow]: Cvjprod of the recorded iterations
    double *zs2prod = nullptr;                   // [nrow][netot][2]
};

struct WaveDev {
    double *norms = nullptr;                     // norm trace
    int64_t norms_cap = 0;
    double *zck = nullptr;                       // [netot][2]
    double *etot = nullptr, *potiflux = nullptr, *zar1flux = nullptr, *reacfct = nullptr;
    int64_t *fl_idx = nullptr, *fl_didx = nullptr;
    int *fl_dptr = nullptr, *fl_dir1 = nullptr, *fl_block = nullptr, *nelebas = nullptr;
    double *zcr = nullptr, *zcdr = nullptr;      // [nflux][netot][2]
    double *zs2 = nullptr, *cvj = nullptr;       // [ncan][nj][nv][netot][2], [ncan][nj][nv]
    double *fd = nullptr;                        // [nelec][nj][nv][npun1]
    int *nobc = nullptr, *r2abs_map = nullptr;
    double *djmmp = nullptr;                     // wave's Djmmp
    double *efe = nullptr, *zfe = nullptr;       // PsiE
    double *psi0 = nullptr;                      // photodissociation (iphoto >= 1): the initial packet
    ProdDev prod;                                // product-state projection, if set
};

// one CTA of the update kernel: a non-empty (segment, point chunk) pair with
// the table entries its prologue needs already resolved, so no CTA starts with
// a chain of dependent loads (48 bytes, three 16-byte loads)
struct alignas(16) UpdChunk {
    long long off;                   // flat offset of the segment
    long long voff;                  // first same-Omega source: its row in the potential tables
    long long poff;                  // first source: flat offset of its psi row (off for the segment itself)
    int seg;
    int chunk_ns;                    // point chunk | number of sources << 8
    int n;                           // stored points of the segment up to the chunk's end
    int wa;                          // wave << 8 | angle
};

struct Ctx {
    mw3_grid grid;
    int n1, n2, na, ne, npt;
    bool fp64;
    std::string err;
    cudaStream_t stream = nullptr;
    int64_t launches = 0;
    bool started = false;
    int64_t it = 0;                  // Chebyshev index of psi_k (all waves advance together)
    int64_t norm_slot = 0;           // iterations recorded since the last start/upload
    // per-iteration Cvj / Cvjprod record (the Cvj.NNNN / Cvjprod.NNNN dumps): a ring
    // of hist_cap iterations at slot norm_slot mod hist_cap, hist_n of them valid
    int64_t hist_cap = 0, hist_n = 0;
    double *d_cvjh = nullptr;        // [hist_cap][G nj nv]

    // host copies of the shared grid
    std::vector<int> npunreal, indr1, indr2;
    std::vector<double> vvv;

    std::vector<WaveTables> waves;
    std::vector<WaveDev> wdev;
    std::vector<ProdTables> prodt;   // per wave (empty or .on = false: no projection)

    // context-wide block list (all waves)
    int G = 0;                       // total blocks
    int64_t NT = 0;                  // total flat points
    bool built = false;              // device tables built for the current wave set

    // shared grid on the device
    int *d_indr1 = nullptr, *d_indr2 = nullptr, *d_npunreal = nullptr;
    double *d_vvv = nullptr;
    int *d_map = nullptr;            // [na][n1][n2] local point index, -1 = not stored
    int *d_mapT = nullptr;           // [na][n2][n1] the same, r1 fastest (stored points are r1-major runs)
    int *d_rows = nullptr;           // [na][n2][4][2]: stored-r1 bits of word w, index of the first point in it
    int *d_rows_ok = nullptr;        // [na]: 1 when every R row's indices run consecutively in r1
    // block tables
    int *d_blk_wave = nullptr, *d_blk_elec = nullptr, *d_blk_om = nullptr;
    int64_t *d_foff = nullptr;       // [G][na] context-wide flat start of (block, angle)
    int *d_cpl = nullptr;            // [G][3][2]: (source block, q) of the l^2 couplings, -1 = none
    int *d_vsrc = nullptr;           // [G][nelec]: same-Omega source blocks of V, -1 = none
    int *d_nopr1 = nullptr;          // [W][na]
    double *d_p2r1 = nullptr, *d_p2r2 = nullptr;     // [W][na][n1], [W][na][n2]
    double *d_absfr1 = nullptr, *d_absfr2 = nullptr; // [W][n1], [W][n2]
    float *d_absfr1f = nullptr, *d_absfr2f = nullptr; // FP32 copies (mixed update)
    int *d_abs_start = nullptr;      // [W][2]: first r1 / R index whose FP32 factor is not 1 (0: not a suffix)
    // recursion vectors (context-wide flat layout), H accumulator, norm partials
    double *d_psiA = nullptr, *d_psiB = nullptr;
    double *d_pk = nullptr, *d_pkm1 = nullptr;       // aliases, swapped every iteration
    double *d_h = nullptr;
    double *d_normpart = nullptr;    // [G*na]
    // per-wave device tables
    int64_t *d_wflat0 = nullptr;     // [W+1]
    int *d_wseg0 = nullptr, *d_wseg1 = nullptr;      // segment range of each wave
    double **d_norm_ptrs = nullptr;  // [W]: norm trace [cap], then <psi0|psi_k> [cap] (photodissociation)
    double *d_autopart = nullptr;    // block partial sums of <psi0|psi_k>
    int auto_nb = 0;                 // their count for the largest photodissociation wave
    int64_t *d_norm_cap = nullptr;   // [W]
    double **d_zfe_ptrs = nullptr;   // [W]
    double *d_zcke = nullptr;        // [W][nofemax][2]
    int nofemax = 0;
    // rectangles of type T (double or float): X = psi, Y = transform scratch
    void *d_X = nullptr, *d_Y = nullptr;
    // DST matrices (type T): S2 [n2][n2]; S1 of every (wave, angle) length, packed
    void *d_S2 = nullptr, *d_S1 = nullptr;
    // FP64 DST along R by Rader's algorithm (npun2 = 256, npun2 + 1 = 257 prime, root 3)
    double2 *d_rd_tw = nullptr;      // W_256^k
    double2 *d_rd_ch = nullptr;      // FFT_256 of the Rader kernel exp(-2 pi i 3^-m / 257), / 256
    short *d_rd_col = nullptr;       // q -> input column 3^q mod 257 - 1
    int *d_rd_out = nullptr;         // p -> output column | (odd output) << 16
    int64_t *d_rowpre = nullptr;     // [G na + 1]: rows ir1 < nopr1 before each segment
    int64_t *d_S1off = nullptr;      // [W][na]
    // explicit angular kinetic matrices (type T)
    void *d_xj2 = nullptr;           // [G][n1][na][na]
    void *d_xl2p = nullptr;          // [G][3][n2][na][na]
    std::vector<char> h_slot_used;   // [G][3]
    // electronic Coriolis coupling of the waves that enable it: the target blocks
    // (ascending), per target up to ec_slots source blocks (-1: none) and the index of
    // each source's channel-pair matrix
    int ec_nt = 0, ec_slots = 0, ec_pairs = 0;
    std::vector<int> h_ec_tgt;       // [ec_nt]
    std::vector<int> h_ec_psrc;      // [ec_pairs] source block of each pair
    int *d_ec_tgt = nullptr, *d_ec_src = nullptr, *d_ec_mat = nullptr;   // [ec_nt], [ec_nt][ec_slots] x2
    double *d_ec_y = nullptr;        // [ec_pairs][n1][na] j-basis scalars
    void *d_xj2e = nullptr;          // [ec_pairs][n1][na][na] channel-pair j^2 matrices
    // inputs of the device-side assembly of xj2/xl2p
    int *d_blk_nojb = nullptr, *d_blk_jbas = nullptr;
    double *d_blk_yj2 = nullptr;
    double *d_djall = nullptr;
    int64_t *d_djoff = nullptr;
    int *d_wnangu2 = nullptr, *d_wj0 = nullptr, *d_winc = nullptr, *d_wiommin = nullptr, *d_wiommax = nullptr,
        *d_wnom = nullptr, *d_wnj2 = nullptr;
    double *d_l2all = nullptr;
    int64_t *d_l2off = nullptr, *d_l2uoff = nullptr;
    char *d_l2used = nullptr;
    // target lists of the angular kernels
    int *d_tj_ptr = nullptr, *d_tj = nullptr;   // per (ir1, chunk of ir2): (a<<20 | ir)
    int *d_tl_ptr = nullptr, *d_tl = nullptr;   // per (ir2, chunk of ir1)
    int *d_quirk_ptr = nullptr, *d_quirk = nullptr;  // per (wave, angle): local points with ir1 > nopr1
    int ncj = 0, ncl = 0;
    int ang_cw = 64;                 // column chunk of the explicit angular kernels (fit_smem)
    int ang_cw_fit = 64;             // the widest chunk whose shared memory fits (set at create)
    // path choices (mw3_set_choices, mw3_autotune); -1 (0 for k_cw) keeps the built-in rule
    int k_dst = -1;                  // radial DST: mixed 0 fused split-FP16, 1 fused 3xTF32, 2 three-kernel
                                     // tensor-core, 3 CUDA-core FP32; FP64 0 folded dense, 1 Rader FFT (npun2 = 256)
    int k_xt = -1;                   // FP32 rectangle stored [R][r1]: 0 no, 1 yes where eligible
    int k_ang = -1;                  // mixed angular terms: 0 explicit kernels, 1 factorised tensor-core kernel
    int k_cw = 0;                    // column chunk of the explicit angular kernels (8..ang_cw_fit, power of 2)
    // scratch for mw3_hphi
    double *d_tmp = nullptr;
    int64_t tmp_cap = 0;
    int nseg = 0;                    // G*na segments, block-major
    int nchunk = 1;                  // point chunks per segment (kPointChunk points each)
    UpdChunk *d_upd_desc = nullptr;  // non-empty (segment, chunk) pairs with their tables resolved
    int n_upd_chunks = 0;
    // context-wide accumulators (all waves share netot, the energy grid, j/v ranges)
    int NF = 0, netot = 0, nj = 0, nv = 0;
    int64_t *d_fl_idx = nullptr, *d_fl_didx = nullptr;
    int *d_fl_dptr = nullptr, *d_fl_dir1 = nullptr;
    double *d_fl_poti = nullptr, *d_zar = nullptr, *d_etot = nullptr, *d_zck = nullptr;
    double *d_fpsi = nullptr;        // [NF][4]: psi, dpsi (re, im)
    // mixed path: the flux samples and C_k(E) of the last kFluxSlots iterations,
    // FP32, slot = iteration mod kFluxSlots; every iteration adds one slice of the
    // flux points over all slots into zCR/zCdR, and everything pending is added
    // before the accumulators are read
    float *d_fring = nullptr;        // [kFluxSlots][NF][3]
    float *d_zar32 = nullptr;        // the r1 derivative row at the flux line, FP32 (mixed path)
    // mixed path: each flux line's derivative terms as runs of consecutive points with
    // consecutive r1 (CSR: fl_rptr[f]..fl_rptr[f+1]), when the runs are long enough
    int *d_fl_rptr = nullptr;
    int4 *d_fl_runs = nullptr;       // (flat index lo, flat index hi, first r1, length)
    bool fl_runs = false;
    float *d_cring = nullptr;        // [kFluxSlots][netot][2]
    int fl_q = 32;                   // a slice of the flux points is flushed every fl_q iterations
    // mixed path: the Cvj projection in FP32 (from the FP32 copy of psi) and Cvj of the
    // last kFluxRing iterations with their C_k(E) (slot = iteration mod kFluxRing),
    // added into zS2 at the iterations = kFluxRing - 1 mod kFluxRing and before every read
    float *d_cvring = nullptr;       // [kFluxRing][G nj nv]
    float *d_cvcring = nullptr;      // [kFluxRing][netot][2]
    float *d_dj32 = nullptr;         // [G][nj][na]: Djmmp columns of the projection, 0 where Cvj is off
    float *d_fd32 = nullptr;         // fd in FP32
    float *d_xj32 = nullptr;         // [G][n1][nj]
    // CUDA graphs of kGraphIters iterations, one per parity of the psi buffers: the
    // kernels read the iteration and the norm slot as d_itbase[0/1] plus the offset
    // captured, so one graph serves every block of iterations
    cudaGraphExec_t graph_exec[2] = {nullptr, nullptr};
    int64_t graph_launches[2] = {0, 0};  // kernel launches one replay stands for
    int64_t *d_itbase = nullptr;
    bool capturing = false;
    int64_t cap_it0 = 0, cap_slot0 = 0;
    bool graphs_off = false;         // MW3_NO_GRAPHS=1, or a capture that failed
    double *d_zcr = nullptr, *d_zcdr = nullptr;          // [NF][netot][2]
    double *d_xj = nullptr;          // [G][n1][nj] angular projection at ir2abs
    double *d_cvj = nullptr;         // [G][nj][nv]
    double *d_zs2 = nullptr;         // [G][nj][nv][netot][2]
    int *d_blk_j00 = nullptr, *d_blk_inc = nullptr, *d_blk_isref = nullptr;
    int *d_r2abs = nullptr;          // [W][na][n1]
    double *d_fd = nullptr;          // [nelec][nj][nv][n1] (shared by the waves)
    int *d_nobc = nullptr;           // [nelec][nj]
    double sah2 = 1.0;
    int jini = 0, jmax = 0, nvini = 0, nvmax = 0, kminelastic = 0, gate_elastic = 0, jref = 0, nvref = 0;
    bool use_tc = true;              // mixed path: radial DSTs on the tensor cores when the shape allows
    // mixed path: factorised angular contraction on the tensor cores (mw3_tc_ang.cu)
    bool use_tc_ang = false;
    float *d_ang_dfw = nullptr, *d_ang_dbk = nullptr;   // [G][2][64*64] Djmmp hi/lo planes, both layouts
    float *d_ang_yj = nullptr;                          // [G][n1][64] yyy(j, r1) by ladder slot
    float *d_ang_l2 = nullptr;                          // [G][3][n2][64] xl2mat_j(Om, Om+q; R)
    int *d_ang_chain_ptr = nullptr, *d_ang_chain = nullptr;   // blocks per (wave, electronic state), Omega ascending
    int *d_ang_tiles = nullptr;                         // 16 r1 x 8 R tiles holding stored points
    int ang_ntiles = 0;
    std::vector<int> ang_wchain;                        // [W+1] first chain of each wave
    // mixed path: the whole radial DST chain in one tensor-core kernel per slab (mw3_tc_dst2d.cu)
    bool use_tc_dst2d = false;
    float *d_dst_planes = nullptr;   // S1 of every length: 128 x 128 TF32 hi/lo chunk planes
    float *d_dst_s2fold = nullptr;   // S2 split by column parity (DST-I symmetry), hi/lo chunk planes
    // the split-FP16 form of the fused DST (default; MW3_DST_TF32=1 keeps the 3xTF32 one):
    // the same planes as FP16 hi/lo x 2^12 in chunks of 32, each slab's largest |X|
    bool dst_f16 = false;
    // the mixed rectangle transposed, [G][na][n2][n1] (r1 fastest): the update and the
    // scatter then store it along the stored points' r1 runs (coalesced); only with
    // the split-FP16 fused DST and the factorised angular contraction, on request
    bool x_t = false;
    void *d_dst_planes16 = nullptr, *d_dst_s2fold16 = nullptr;
    int64_t *d_dst_s1off16 = nullptr;
    unsigned *d_xmax = nullptr;      // [G na], written by the scatter and update kernels
    int64_t *d_dst_s1off = nullptr;  // [W][na] float offset of the slab's S1
    float *d_p2r1f = nullptr, *d_p2r2f = nullptr;      // FP32 copies of the momenta tables
    alignas(64) unsigned char dst_xmap[128] = {};       // TMA map of the rectangles (CUtensorMap)
    // mixed path with the fused DSTs: H psi (without V) kept in FP32, and the
    // potential pre-scaled for the update: vr = V 2/delta2 - [same state] emindlt 2/delta2
    bool h32 = false;
    float *d_h32 = nullptr;          // [NT]
    float *d_vr32 = nullptr;         // like vvv, FP32 (mixed update)
    float *d_pk32 = nullptr, *d_pkm1_32 = nullptr;   // FP32 copies of psi_k and of the next psi (mixed update)
    int *d_tc_err = nullptr;         // set by a tensor-core kernel whose mbarrier wait ran out
    int *h_flag = nullptr;           // pinned copy of it, read in the context's stream
    // optional per-stage event timing (mw3_profile)
    bool prof = false;
    std::vector<cudaEvent_t> prof_ev;    // (MW3_NSTAGES+1) events per recorded iteration
    int64_t prof_n = 0, prof_cap = 0;
    std::vector<void *> allocs;      // everything allocated for the wave set
};

// device-side view of the shared grid and block tables (passed by value)
struct DevGrid {
    int n1, n2, na, ne, npt, G;
    const int *indr1, *indr2, *npunreal;
    const double *vvv;
    const int *map;
    const int *mapT;
    const int64_t *foff;
    const int *blk_wave, *blk_elec, *blk_om;
    int xt;                          // rectangle layout: 0 [..][r1][R], 1 [..][R][r1]
};

inline DevGrid devgrid(Ctx &c)
{
    DevGrid d;
    d.n1 = c.n1; d.n2 = c.n2; d.na = c.na; d.ne = c.ne; d.npt = c.npt; d.G = c.G;
    d.indr1 = c.d_indr1; d.indr2 = c.d_indr2; d.npunreal = c.d_npunreal; d.vvv = c.d_vvv;
    d.map = c.d_map; d.mapT = c.d_mapT; d.foff = c.d_foff;
    d.blk_wave = c.d_blk_wave; d.blk_elec = c.d_blk_elec; d.blk_om = c.d_blk_om;
    d.xt = c.x_t ? 1 : 0;
    return d;
}

// tensor-core radial DSTs of the mixed path (mw3_tc.cu); false = shape not supported
bool tc_dst_supported(Ctx &c);
void launch_tc_dst(Ctx &c, const float *X, float *Y, double *H, int g_begin, int g_end, int stage_base);
// tensor-core angular terms of the mixed path (mw3_tc_ang.cu); sets c.use_tc_ang
int build_tc_ang(Ctx &c);
void launch_tc_ang(Ctx &c, const float *X, double *H, int g_begin, int g_end, bool xt);
void launch_tc_ang(Ctx &c, const float *X, float *H, int g_begin, int g_end, bool xt);
// fused tensor-core radial DSTs of the mixed path (mw3_tc_dst2d.cu); sets c.use_tc_dst2d
int build_tc_dst2d(Ctx &c);
// true when the environment asks for the general (indexed) tables even where the
// stored points form regular lines (MW3_GENERAL_TABLES=1; for tests)
inline bool general_tables()
{
    const char *v = std::getenv("MW3_GENERAL_TABLES");
    return v && v[0] == '1';
}
// the TMA tensor map of the rectangles (after they are allocated)
int encode_tc_dst2d_xmap(Ctx &c);
// the [R][r1] rectangle is possible: fused split-FP16 DST and factorised angular kernel,
// no electronic Coriolis coupling, n1 a multiple of 4 and at least 32
bool xt_eligible(const Ctx &c);
void launch_tc_dst2d(Ctx &c, const float *X, float *H, int g_begin, int g_end);
std::vector<double> dst_matrix(int n);

// ---------------------------------------------------------------------------
// setup (mw3_setup.cu)
// ---------------------------------------------------------------------------
int build_wave_tables(Ctx &c, const mw3_wave &w, WaveTables &t, std::string &err);
void ecor_pairs(const Ctx &c, const WaveTables &t, std::vector<int> &src, std::vector<int> &dst,
                std::vector<double> &y);
int noptfft(int nin, int ntot);
void riccati_fg(int l, double x, double *f, double *g);

// ---------------------------------------------------------------------------
// kernels (mw3_kernels.cu)
// ---------------------------------------------------------------------------
template <typename T>
void launch_scatter(Ctx &c, const double *psi, float *psi32, int g_begin, int g_end);
template <typename T>
void launch_hphi(Ctx &c, const double *psi, int g_begin, int g_end);
void launch_fill_pattern(Ctx &c, double *p, int64_t n);
// records the boundary event of a stage when per-stage timing is on
void stage_mark(Ctx &c, int stage);
template <typename T>
void launch_update(Ctx &c, int first);
template <typename T>
void launch_build_kinetic(Ctx &c);
void launch_accumulators(Ctx &c, int64_t it);
// mixed path: add the pending ring slots to the FP64 flux accumulators
void flush_flux(Ctx &c);
void flush_cvj(Ctx &c);
// the FP32 Djmmp columns of the Cvj projection (mixed path), once the tables are on the device
void build_cvj32(Ctx &c);
constexpr int kFluxRing = 32;       // Cvj ring: iterations between its flushes
constexpr int kFluxSlots = 128;     // flux ring: iterations in each accumulated sum
void launch_norms(Ctx &c, int64_t slot);
// writes the context's iteration and norm slot where a graph replay reads them
void launch_set_itbase(Ctx &c);
// prodpaq + prodcvj of every wave that has a product projection
void launch_product(Ctx &c);
// check's autocorrelation <psi0|psi_k> of every photodissociation wave into slot
void launch_autocorr(Ctx &c, int64_t slot);
// funE's C_k(E) for iteration it (launched before the update that uses it)
void launch_fe_coef(Ctx &c, int64_t it);
// the iteration's Cvj (and Cvjprod) into the history ring at slot mod hist_cap
void launch_cvj_keep(Ctx &c, int64_t it, int64_t slot);
constexpr int kGraphIters = 32;      // iterations per captured graph (one ring cycle)
static_assert(kFluxRing == kGraphIters, "a captured block must cycle the Cvj ring exactly once");
static_assert(kGraphIters % (kFluxSlots / 4) == 0, "flux slice flushes must repeat with the captured block");
void launch_addv(Ctx &c, const double *psi, int g0, int g1);
void launch_totalflux(Ctx &c, int w, double *d_out, double *d_outelec);
void set_kernel_attributes(Ctx &c);
// picks c.ang_cw so that every kernel's dynamic shared memory fits optin bytes
bool fit_smem(Ctx &c, size_t optin);
// the C-ABI's error reporting: a failed launch (cudaGetLastError), and after a
// synchronisation the tensor-core kernels' wait-timeout flag
int api_check_launch(Ctx &c, const char *where);
int api_check_device_flags(Ctx &c, const char *where);

}  // namespace mw3

// the opaque handle of the C-ABI
struct mw3_ctx {
    mw3::Ctx c;
};

#define MW3_CUDA_TRY(expr)                                                            \
    do {                                                                              \
        cudaError_t e_ = (expr);                                                      \
        if (e_ != cudaSuccess) {                                                      \
            c.err = std::string(#expr) + ": " + cudaGetErrorString(e_);               \
            return MW3_ERR_CUDA;                                                      \
        }                                                                             \
    } while (0)
