// C-ABI of libmw3gpu (include/mw3gpu.h): context management, device-side
// assembly of the per-wave tables and the Chebyshev driver loop
// (SRC/main_madwave3.f:238-368 for one process, every partial wave of the
// context advancing together).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <new>

#include "mw3_internal.h"

using mw3::Ctx;
using mw3::WaveDev;
using mw3::WaveTables;

namespace {


template <typename V>
int dupload(Ctx &c, V **dst, const V *src, size_t n)
{
    *dst = nullptr;
    size_t bytes = sizeof(V) * std::max<size_t>(n, 1);
    cudaError_t e = cudaMalloc((void **)dst, bytes);
    if (e != cudaSuccess) {
        c.err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
        return MW3_ERR_NOMEM;
    }
    c.allocs.push_back(*dst);
    if (n && src) {
        e = cudaMemcpy(*dst, src, sizeof(V) * n, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            c.err = std::string("cudaMemcpy: ") + cudaGetErrorString(e);
            return MW3_ERR_CUDA;
        }
    }
    return MW3_OK;
}

template <typename V>
int dupload(Ctx &c, V **dst, const std::vector<V> &v)
{
    return dupload(c, dst, v.data(), v.size());
}

template <typename V>
int dalloc(Ctx &c, V **dst, size_t n, bool zero = true)
{
    int rc = dupload<V>(c, dst, nullptr, n);
    if (rc) return rc;
    if (zero) {
        cudaError_t e = cudaMemset(*dst, 0, sizeof(V) * std::max<size_t>(n, 1));
        if (e != cudaSuccess) {
            c.err = std::string("cudaMemset: ") + cudaGetErrorString(e);
            return MW3_ERR_CUDA;
        }
    }
    return MW3_OK;
}

void free_device(Ctx &c)
{
    for (int p = 0; p < 2; p++) {
        if (c.graph_exec[p]) cudaGraphExecDestroy(c.graph_exec[p]);
        c.graph_exec[p] = nullptr;
        c.graph_launches[p] = 0;
    }
    c.d_itbase = nullptr;
    for (void *p : c.allocs) cudaFree(p);
    c.allocs.clear();
    c.built = false;
}

#define TRY(x)                 \
    do {                       \
        int rc_ = (x);         \
        if (rc_) return rc_;   \
    } while (0)

}  // namespace

namespace mw3 {
// DST-I matrix of length n, the unnormalised RODFT00 of FFTW: S[i][k] = 2 sin(pi (i+1)(k+1)/(n+1))
std::vector<double> dst_matrix(int n)
{
    std::vector<double> s((size_t)n * n);
    const double pi = 3.14159265358979323846;
    for (int i = 0; i < n; i++)
        for (int k = 0; k < n; k++) {
            long long m = ((long long)(i + 1) * (k + 1)) % (2LL * (n + 1));
            s[(size_t)i * n + k] = 2.0 * sin(pi * (double)m / (double)(n + 1));
        }
    return s;
}
}  // namespace mw3

namespace {
using mw3::dst_matrix;

template <typename T>
std::vector<T> cast(const std::vector<double> &v)
{
    return std::vector<T>(v.begin(), v.end());
}

template <typename T>
int build_typed(Ctx &c)
{
    int na = c.na, n1 = c.n1, n2 = c.n2;
    int W = (int)c.waves.size();
    // DST matrices
    {
        std::vector<T> s2 = cast<T>(dst_matrix(n2));
        T *d;
        TRY(dupload(c, &d, s2));
        c.d_S2 = d;
        std::map<int, int64_t> off;
        std::vector<T> s1all;
        std::vector<int64_t> s1off((size_t)W * na);
        for (int w = 0; w < W; w++)
            for (int a = 0; a < na; a++) {
                int nn = c.waves[w].nopr1[a];
                auto it = off.find(nn);
                if (it == off.end()) {
                    int64_t o = (int64_t)s1all.size();
                    std::vector<T> m = cast<T>(dst_matrix(nn));
                    s1all.insert(s1all.end(), m.begin(), m.end());
                    it = off.emplace(nn, o).first;
                }
                s1off[(size_t)w * na + a] = it->second;
            }
        T *d1;
        TRY(dupload(c, &d1, s1all));
        c.d_S1 = d1;
        TRY(dupload(c, &c.d_S1off, s1off));
    }
    // rectangles, zero outside the stored points
    size_t rect = (size_t)c.G * na * n1 * n2;
    T *x, *y;
    TRY(dalloc(c, &x, rect));
    TRY(dalloc(c, &y, rect));
    c.d_X = x;
    c.d_Y = y;
    // channel-pair j^2 matrices of the electronic Coriolis variant (every path)
    c.d_xj2e = nullptr;
    if (c.ec_pairs > 0) {
        T *xe;
        TRY(dalloc(c, &xe, (size_t)c.ec_pairs * n1 * na * na));
        c.d_xj2e = xe;
    }
    // explicit angular matrices (not needed when the factorised contraction runs)
    c.d_xj2 = c.d_xl2p = nullptr;
    if (c.use_tc_ang) {
        mw3::launch_build_kinetic<T>(c);
        return MW3_OK;
    }
    T *xj2, *xl2p;
    TRY(dalloc(c, &xj2, (size_t)c.G * n1 * na * na));
    TRY(dalloc(c, &xl2p, (size_t)c.G * 3 * n2 * na * na));
    c.d_xj2 = xj2;
    c.d_xl2p = xl2p;
    mw3::launch_build_kinetic<T>(c);
    return MW3_OK;
}

// cudaFree one of the context's allocations and drop it from the list
void dfree(Ctx &c, void *p)
{
    if (!p) return;
    for (size_t i = 0; i < c.allocs.size(); i++)
        if (c.allocs[i] == p) {
            cudaFree(p);
            c.allocs.erase(c.allocs.begin() + (long)i);
            return;
        }
}

// the Cvj / Cvjprod history ring for hist_cap iterations (none when 0)
int alloc_history(Ctx &c)
{
    dfree(c, c.d_cvjh);
    c.d_cvjh = nullptr;
    for (auto &w : c.wdev) {
        dfree(c, w.prod.cvjph);
        w.prod.cvjph = nullptr;
    }
    c.hist_n = 0;
    if (c.hist_cap <= 0) return MW3_OK;
    if (c.n2 > 1) TRY(dalloc(c, &c.d_cvjh, (size_t)c.hist_cap * c.G * c.nj * c.nv));
    for (auto &w : c.wdev)
        if (w.prod.cvjprod) TRY(dalloc(c, &w.prod.cvjph, (size_t)c.hist_cap * w.prod.nrow));
    return MW3_OK;
}

int build_device(Ctx &c)
{
    if (c.built) return MW3_OK;
    if (c.waves.empty()) {
        c.err = "no partial wave added";
        return MW3_ERR_STATE;
    }
    free_device(c);
    int na = c.na, n1 = c.n1, n2 = c.n2, ne = c.ne;
    int W = (int)c.waves.size();
    c.ang_cw = c.k_cw > 0 ? c.k_cw : c.ang_cw_fit;
    // ---- shared grid ----
    TRY(dupload(c, &c.d_indr1, c.indr1));
    TRY(dupload(c, &c.d_indr2, c.indr2));
    TRY(dupload(c, &c.d_npunreal, c.npunreal));
    TRY(dupload(c, &c.d_vvv, c.vvv));
    {
        std::vector<int> map((size_t)na * n1 * n2, -1);
        for (int a = 0; a < na; a++)
            for (int ir = 0; ir < c.npunreal[a]; ir++) {
                int ir1 = c.indr1[(size_t)a * c.npt + ir] - 1, ir2 = c.indr2[(size_t)a * c.npt + ir] - 1;
                map[((size_t)a * n1 + ir1) * n2 + ir2] = ir;
            }
        TRY(dupload(c, &c.d_map, map));
        std::vector<int> mapT((size_t)na * n1 * n2);
        for (int a = 0; a < na; a++)
            for (int i1 = 0; i1 < n1; i1++)
                for (int i2 = 0; i2 < n2; i2++)
                    mapT[((size_t)a * n2 + i2) * n1 + i1] = map[((size_t)a * n1 + i1) * n2 + i2];
        TRY(dupload(c, &c.d_mapT, mapT));
        // each (angle, R) row's stored points by r1 word w < 4 (r1 < 128, the fused DST's
        // range): the bits of the stored r1 and the index of the row's first point at or
        // after r1 = 32 w, so a point's index is that plus the bits below it; an angle
        // qualifies when every row's indices run consecutively in r1 order (points
        // stored R outer, r1 inner)
        std::vector<int> rows((size_t)na * n2 * 4 * 2, 0), rows_ok(na, 1);
        for (int a = 0; a < na; a++)
            for (int i2 = 0; i2 < n2; i2++) {
                int base = -1, k = 0;
                for (int i1 = 0; i1 < n1; i1++) {
                    const int idx = map[((size_t)a * n1 + i1) * n2 + i2];
                    if (idx < 0) continue;
                    if (base < 0) base = idx;
                    if (idx != base + k) rows_ok[a] = 0;
                    k++;
                }
                int before = base < 0 ? 0 : base;
                for (int w = 0; w < 4; w++) {
                    unsigned bits = 0u;
                    for (int b = 0; b < 32 && 32 * w + b < n1; b++)
                        if (map[((size_t)a * n1 + 32 * w + b) * n2 + i2] >= 0) bits |= 1u << b;
                    rows[(((size_t)a * n2 + i2) * 4 + w) * 2] = (int)bits;
                    rows[(((size_t)a * n2 + i2) * 4 + w) * 2 + 1] = before;
                    before += __builtin_popcount(bits);
                }
            }
        TRY(dupload(c, &c.d_rows, rows));
        TRY(dupload(c, &c.d_rows_ok, rows_ok));
    }
    // ---- layout of the wave set ----
    int G = 0;
    int64_t NT = 0;
    for (auto &t : c.waves) {
        t.g0 = G;
        t.flat0 = NT;
        G += t.ncan;
        NT += t.ntot;
    }
    c.G = G;
    c.NT = NT;
    c.nseg = G * na;
    std::vector<int> bw(G), be(G), bo(G), bnoj(G), bjb((size_t)G * na);
    std::vector<int64_t> foff((size_t)G * na);
    std::vector<int> cpl((size_t)G * 6, -1), vsrc((size_t)G * ne, -1);
    std::vector<double> byj2((size_t)G * n1 * na);
    c.h_slot_used.assign((size_t)G * 3, 0);
    std::vector<int64_t> wflat0(W + 1);
    std::vector<int> wseg0(W), wseg1(W);
    for (int w = 0; w < W; w++) {
        WaveTables &t = c.waves[w];
        wflat0[w] = t.flat0;
        wseg0[w] = t.g0 * na;
        wseg1[w] = (t.g0 + t.ncan) * na;
        for (int b = 0; b < t.ncan; b++) {
            int g = t.g0 + b;
            bw[g] = w;
            be[g] = t.nelebas[b];
            bo[g] = t.iombas[b];
            bnoj[g] = t.nojbas[b];
            for (int k = 0; k < na; k++) bjb[(size_t)g * na + k] = t.jbas[(size_t)b * na + k];
            for (int a = 0; a < na; a++) foff[(size_t)g * na + a] = t.flat0 + t.offs[(size_t)a * t.ncan + b];
            std::copy(t.yj2.begin() + (size_t)b * n1 * na, t.yj2.begin() + (size_t)(b + 1) * n1 * na,
                      byj2.begin() + (size_t)g * n1 * na);
            int nv = 0;
            for (int s = 0; s < t.ncan; s++) {
                if (t.iombas[s] == t.iombas[b] && nv < ne) vsrc[(size_t)g * ne + nv++] = t.g0 + s;
                if (t.nelebas[s] == t.nelebas[b] && abs(t.iombas[s] - t.iombas[b]) <= 1) {
                    int q = t.iombas[s] - t.iombas[b];
                    cpl[((size_t)g * 3 + (q + 1)) * 2] = t.g0 + s;
                    cpl[((size_t)g * 3 + (q + 1)) * 2 + 1] = q;
                    c.h_slot_used[(size_t)(t.g0 + s) * 3 + (q + 1)] = 1;
                }
            }
        }
    }
    wflat0[W] = NT;
    TRY(dupload(c, &c.d_blk_wave, bw));
    TRY(dupload(c, &c.d_blk_elec, be));
    TRY(dupload(c, &c.d_blk_om, bo));
    TRY(dupload(c, &c.d_blk_nojb, bnoj));
    TRY(dupload(c, &c.d_blk_jbas, bjb));
    TRY(dupload(c, &c.d_blk_yj2, byj2));
    TRY(dupload(c, &c.d_foff, foff));
    TRY(dupload(c, &c.d_cpl, cpl));
    TRY(dupload(c, &c.d_vsrc, vsrc));
    TRY(dupload(c, &c.d_wflat0, wflat0));
    TRY(dupload(c, &c.d_wseg0, wseg0));
    TRY(dupload(c, &c.d_wseg1, wseg1));
    // ---- electronic Coriolis pairs (waves with the variant on) ----
    {
        std::vector<int> tg, psrc;
        std::vector<std::vector<std::pair<int, int>>> srcs;   // per target: (source block, pair)
        std::vector<double> yall;
        for (int w = 0; w < W; w++) {
            const WaveTables &t = c.waves[w];
            std::vector<int> s, d;
            std::vector<double> y;
            ecor_pairs(c, t, s, d, y);
            for (size_t p = 0; p < s.size(); p++) {
                int gs = t.g0 + s[p], gd = t.g0 + d[p];
                if (tg.empty() || tg.back() != gd) {
                    tg.push_back(gd);
                    srcs.emplace_back();
                }
                srcs.back().emplace_back(gs, (int)psrc.size());
                psrc.push_back(gs);
            }
            yall.insert(yall.end(), y.begin(), y.end());
        }
        int slots = 0;
        for (auto &v : srcs) slots = std::max(slots, (int)v.size());
        c.ec_nt = (int)tg.size();
        c.ec_slots = slots;
        c.ec_pairs = (int)psrc.size();
        c.h_ec_tgt = tg;
        c.h_ec_psrc = psrc;
        c.d_ec_tgt = c.d_ec_src = c.d_ec_mat = nullptr;
        c.d_ec_y = nullptr;
        if (c.ec_nt > 0) {
            std::vector<int> es((size_t)c.ec_nt * slots, -1), em((size_t)c.ec_nt * slots, -1);
            for (int q = 0; q < c.ec_nt; q++)
                for (size_t k = 0; k < srcs[q].size(); k++) {
                    es[(size_t)q * slots + k] = srcs[q][k].first;
                    em[(size_t)q * slots + k] = srcs[q][k].second;
                }
            TRY(dupload(c, &c.d_ec_tgt, tg));
            TRY(dupload(c, &c.d_ec_src, es));
            TRY(dupload(c, &c.d_ec_mat, em));
            TRY(dupload(c, &c.d_ec_y, yall));
        }
    }
    // ---- per-wave tables concatenated ----
    std::vector<int> nopr1((size_t)W * na);
    std::vector<double> p2r1((size_t)W * na * n1), p2r2((size_t)W * na * n2), a1((size_t)W * n1),
        a2((size_t)W * n2);
    std::vector<double> djall, l2all;
    std::vector<char> l2used;
    std::vector<int64_t> djoff(W), l2off(W), l2uoff(W);
    std::vector<int> wn2(W), wj0(W), winc(W), wmin(W), wmax(W), wnom(W), wnj2(W);
    std::vector<int> qptr((size_t)W * na + 1, 0), qlist;
    for (int w = 0; w < W; w++) {
        WaveTables &t = c.waves[w];
        std::copy(t.nopr1.begin(), t.nopr1.end(), nopr1.begin() + (size_t)w * na);
        std::copy(t.p2r1.begin(), t.p2r1.end(), p2r1.begin() + (size_t)w * na * n1);
        std::copy(t.p2r2.begin(), t.p2r2.end(), p2r2.begin() + (size_t)w * na * n2);
        std::copy(t.absfr1.begin(), t.absfr1.end(), a1.begin() + (size_t)w * n1);
        std::copy(t.absfr2.begin(), t.absfr2.end(), a2.begin() + (size_t)w * n2);
        djoff[w] = (int64_t)djall.size();
        djall.insert(djall.end(), t.djmmp.begin(), t.djmmp.end());
        l2off[w] = (int64_t)l2all.size();
        l2all.insert(l2all.end(), t.l2tab.begin(), t.l2tab.end());
        l2uoff[w] = (int64_t)l2used.size();
        l2used.insert(l2used.end(), t.l2used.begin(), t.l2used.end());
        wn2[w] = t.nangu2; wj0[w] = t.j0; winc[w] = t.inc; wmin[w] = t.iommin; wmax[w] = t.iommax;
        wnom[w] = t.nom; wnj2[w] = t.nj2;
        for (int a = 0; a < na; a++) {
            for (int ir = 0; ir < c.npunreal[a]; ir++)
                if (c.indr1[(size_t)a * c.npt + ir] > t.nopr1[a]) qlist.push_back(ir);
            qptr[(size_t)w * na + a + 1] = (int)qlist.size();
        }
    }
    TRY(dupload(c, &c.d_nopr1, nopr1));
    {
        // the rows each segment transforms (ir1 < nopr1), as a prefix over segments
        std::vector<int64_t> pre((size_t)G * na + 1, 0);
        for (int s = 0; s < G * na; s++) pre[s + 1] = pre[s] + nopr1[(size_t)bw[s / na] * na + s % na];
        TRY(dupload(c, &c.d_rowpre, pre));
    }
    c.d_rd_tw = c.d_rd_ch = nullptr;
    c.d_rd_col = nullptr;
    c.d_rd_out = nullptr;
    if (n2 == 256 && !(c.fp64 && c.k_dst == 0)) {
        // Rader's tables for the 257-point transform behind the FP64 DST along R: with g = 3
        // a primitive root of 257, W_{g^-p} = sum_q a_q d_{p-q}, a_q = w_{g^q}, d_m =
        // exp(-2 pi i g^-m / 257), a 256-point cyclic convolution; d's FFT / 256 in long double
        const int NP = 257, M = 256;
        std::vector<int> perm(M);
        for (int q = 0, v = 1; q < M; q++, v = (v * 3) % NP) perm[q] = v;
        std::vector<short> col(M);
        std::vector<int> outc(M);
        for (int q = 0; q < M; q++) col[q] = (short)(perm[q] - 1);
        for (int p = 0; p < M; p++) {
            const int j = perm[(M - p) % M];            // W_j lands at convolution index p
            outc[p] = j <= 128 ? 2 * j - 1 : (2 * j - 258) | (1 << 16);
        }
        const long double twopi = 6.283185307179586476925286766559005768L;
        std::vector<double2> tw(M), ch(M);
        for (int k = 0; k < M; k++) {
            const long double th = twopi * (long double)k / M;
            tw[k] = make_double2((double)cosl(th), (double)-sinl(th));
            long double re = 0.0L, im = 0.0L;
            for (int m = 0; m < M; m++) {
                const long double ph = twopi * ((long double)perm[(M - m) % M] / NP + (long double)((m * k) % M) / M);
                re += cosl(ph);
                im -= sinl(ph);
            }
            ch[k] = make_double2((double)(re / M), (double)(im / M));
        }
        TRY(dupload(c, &c.d_rd_tw, tw));
        TRY(dupload(c, &c.d_rd_ch, ch));
        TRY(dupload(c, &c.d_rd_col, col));
        TRY(dupload(c, &c.d_rd_out, outc));
    }
    TRY(dupload(c, &c.d_p2r1, p2r1));
    TRY(dupload(c, &c.d_p2r2, p2r2));
    TRY(dupload(c, &c.d_absfr1, a1));
    TRY(dupload(c, &c.d_absfr2, a2));
    {
        std::vector<float> f1(a1.begin(), a1.end()), f2(a2.begin(), a2.end());
        TRY(dupload(c, &c.d_absfr1f, f1));
        TRY(dupload(c, &c.d_absfr2f, f2));
        // where each wave's absorbers start: the points before both starts have factor
        // 1 exactly, so the update need not read the tables there; an absorber that is
        // not a suffix of its axis gets start 0 (always read)
        const int nw = (int)c.waves.size();
        std::vector<int> st((size_t)nw * 2, 0);
        for (int w = 0; w < nw; w++)
            for (int ax = 0; ax < 2; ax++) {
                const std::vector<float> &f = ax == 0 ? f1 : f2;
                const int n = ax == 0 ? n1 : n2;
                int first = n;
                for (int i = 0; i < n; i++)
                    if (f[(size_t)w * n + i] != 1.0f) {
                        first = i;
                        break;
                    }
                bool suffix = true;
                for (int i = first; i < n; i++) suffix = suffix && f[(size_t)w * n + i] != 1.0f;
                st[(size_t)w * 2 + ax] = suffix ? first : 0;
            }
        TRY(dupload(c, &c.d_abs_start, st));
    }
    TRY(dupload(c, &c.d_djall, djall));
    TRY(dupload(c, &c.d_djoff, djoff));
    TRY(dupload(c, &c.d_l2all, l2all));
    TRY(dupload(c, &c.d_l2off, l2off));
    TRY(dupload(c, &c.d_l2used, l2used));
    TRY(dupload(c, &c.d_l2uoff, l2uoff));
    TRY(dupload(c, &c.d_wnangu2, wn2));
    TRY(dupload(c, &c.d_wj0, wj0));
    TRY(dupload(c, &c.d_winc, winc));
    TRY(dupload(c, &c.d_wiommin, wmin));
    TRY(dupload(c, &c.d_wiommax, wmax));
    TRY(dupload(c, &c.d_wnom, wnom));
    TRY(dupload(c, &c.d_wnj2, wnj2));
    TRY(dupload(c, &c.d_quirk_ptr, qptr));
    TRY(dupload(c, &c.d_quirk, qlist));
    // ---- target lists of the angular kernels ----
    {
        const int kAngCW = c.ang_cw;
        c.ncj = (n2 + kAngCW - 1) / kAngCW;
        c.ncl = (n1 + kAngCW - 1) / kAngCW;
        std::vector<std::vector<int>> bj((size_t)n1 * c.ncj), bl((size_t)n2 * c.ncl);
        for (int a = 0; a < na; a++)
            for (int ir = 0; ir < c.npunreal[a]; ir++) {
                int ir1 = c.indr1[(size_t)a * c.npt + ir] - 1, ir2 = c.indr2[(size_t)a * c.npt + ir] - 1;
                int ent = (a << 20) | ir;
                bj[(size_t)ir1 * c.ncj + ir2 / kAngCW].push_back(ent);
                bl[(size_t)ir2 * c.ncl + ir1 / kAngCW].push_back(ent);
            }
        auto flatten = [](std::vector<std::vector<int>> &b, std::vector<int> &ptr, std::vector<int> &lst) {
            ptr.assign(b.size() + 1, 0);
            for (size_t i = 0; i < b.size(); i++) {
                lst.insert(lst.end(), b[i].begin(), b[i].end());
                ptr[i + 1] = (int)lst.size();
            }
        };
        std::vector<int> pj, lj, pl, ll;
        flatten(bj, pj, lj);
        flatten(bl, pl, ll);
        TRY(dupload(c, &c.d_tj_ptr, pj));
        TRY(dupload(c, &c.d_tj, lj));
        TRY(dupload(c, &c.d_tl_ptr, pl));
        TRY(dupload(c, &c.d_tl, ll));
    }
    // ---- recursion vectors and scratch ----
    TRY(dalloc(c, &c.d_psiA, NT));
    TRY(dalloc(c, &c.d_psiB, NT));
    c.d_pk = c.d_psiA;
    c.d_pkm1 = c.d_psiB;
    TRY(dalloc(c, &c.d_h, NT));
    TRY(dalloc(c, &c.d_tmp, NT));
    c.tmp_cap = NT;
    TRY(dalloc(c, &c.d_tc_err, 1));
    c.nchunk = (c.npt + 1023) / 1024;
    if (c.nchunk > 256) {
        c.err = "more than 256 x 1024 stored points in one angle";
        return MW3_ERR_UNSUPPORTED;
    }
    {
        std::vector<mw3::UpdChunk> ch;
        for (int seg = 0; seg < c.nseg; seg++) {
            int g = seg / na, a = seg % na, ns = 0;
            long long voff = -1, poff = -1;
            for (int q = 0; q < ne; q++) {
                int sb = vsrc[(size_t)g * ne + q];
                if (sb < 0) continue;
                if (ns == 0) {
                    voff = ((((long long)(be[g] - 1) * ne + (be[sb] - 1)) * na) + a) * c.npt;
                    poff = foff[(size_t)sb * na + a];
                }
                ns++;
            }
            for (int k = 0; k * 1024 < c.npunreal[a]; k++)
                ch.push_back(mw3::UpdChunk{foff[seg], voff, poff, seg, k | (ns << 8),
                                      std::min(c.npunreal[a], (k + 1) * 1024), (bw[g] << 8) | a});
        }
        if (ch.empty()) ch.push_back(mw3::UpdChunk{0, -1, -1, 0, 0, 0, 0});
        c.n_upd_chunks = (int)ch.size();
        TRY(dupload(c, &c.d_upd_desc, ch));
    }
    TRY(dalloc(c, &c.d_normpart, (size_t)c.nseg * c.nchunk));
    // ---- accumulators: context-wide arrays, each wave a slice ----
    {
        const WaveTables &t0 = c.waves[0];
        for (auto &t : c.waves)
            if (t.netot != t0.netot || t.ekinmin != t0.ekinmin || t.ekinmax != t0.ekinmax || t.jini != t0.jini ||
                t.jmax != t0.jmax || t.nvini != t0.nvini || t.nvmax != t0.nvmax || t.kminelastic != t0.kminelastic ||
                t.iprod != t0.iprod || t.iphoto != t0.iphoto || t.jref != t0.jref || t.nvref != t0.nvref ||
                t.r1flux_ang != t0.r1flux_ang || t.fd != t0.fd || t.nobc != t0.nobc) {
                c.err = "the partial waves of one context must share the energy grid, j/v ranges, flux line and "
                        "diatomic functions";
                return MW3_ERR_ARG;
            }
        c.netot = t0.netot;
        c.nj = t0.nj;
        c.nv = t0.nv;
        c.jini = t0.jini; c.jmax = t0.jmax; c.nvini = t0.nvini; c.nvmax = t0.nvmax;
        c.kminelastic = t0.kminelastic; c.jref = t0.jref; c.nvref = t0.nvref;
        c.gate_elastic = (t0.iphoto == 0) ? 1 : 0;
        double ah2 = (c.grid.rfin2 - c.grid.rmis2) / (double)(n2 - 1);
        c.sah2 = sqrt(ah2);
        std::vector<int64_t> fidx, fdidx;
        std::vector<int> fdptr, fdir1, bj00(G), binc(G), bref(G), r2abs((size_t)W * na * n1);
        std::vector<double> fpoti;
        int64_t nf = 0;
        for (int w = 0; w < W; w++) {
            WaveTables &t = c.waves[w];
            for (int f = 0; f < t.nflux; f++) {
                fidx.push_back(t.flat0 + t.fl_idx[f]);
                fpoti.push_back(t.flux_gate ? t.potiflux[f] : -1.0e300);
                fdptr.push_back((int)fdidx.size());
                for (int q = t.fl_dptr[f]; q < t.fl_dptr[f + 1]; q++) {
                    fdidx.push_back(t.flat0 + t.fl_didx[q]);
                    fdir1.push_back(t.fl_dir1[q]);
                }
            }
            nf += t.nflux;
            for (int b = 0; b < t.ncan; b++) {
                bj00[t.g0 + b] = t.j00[b];
                binc[t.g0 + b] = t.inc;
                bref[t.g0 + b] = (t.iomref < 0 || b == t.icanref) ? 1 : 0;
            }
            std::copy(t.r2abs_map.begin(), t.r2abs_map.end(), r2abs.begin() + (size_t)w * na * n1);
        }
        fdptr.push_back((int)fdidx.size());
        c.NF = (int)nf;
        // the stored points run along r1 for each R (ir2 outer, ir1 inner), so a flux
        // line's derivative terms are a few runs of consecutive points and r1 (one per
        // valley the potential cut leaves); the mixed path reads runs when they are long
        // enough.  MW3_GENERAL_TABLES=1 keeps the indexed form, so tests can compare both.
        std::vector<int> frptr;
        std::vector<int4> fruns;
        for (int64_t f = 0; f < nf; f++) {
            frptr.push_back((int)fruns.size());
            for (int q = fdptr[f]; q < fdptr[f + 1]; q++) {
                if (q > fdptr[f] && fdidx[q] == fdidx[q - 1] + 1 && fdir1[q] == fdir1[q - 1] + 1) {
                    fruns.back().w++;
                } else {
                    const unsigned long long i = (unsigned long long)fdidx[q];
                    fruns.push_back(make_int4((int)(unsigned)(i & 0xFFFFFFFFull), (int)(unsigned)(i >> 32), fdir1[q], 1));
                }
            }
        }
        frptr.push_back((int)fruns.size());
        c.fl_runs = !c.fp64 && !mw3::general_tables() && !fruns.empty() && fdidx.size() >= 8 * fruns.size();
        c.d_fl_rptr = nullptr;
        c.d_fl_runs = nullptr;
        if (c.fl_runs) {
            TRY(dupload(c, &c.d_fl_rptr, frptr));
            TRY(dupload(c, &c.d_fl_runs, fruns));
        }
        TRY(dupload(c, &c.d_fl_idx, fidx));
        TRY(dupload(c, &c.d_fl_poti, fpoti));
        TRY(dupload(c, &c.d_fl_dptr, fdptr));
        TRY(dupload(c, &c.d_fl_didx, fdidx));
        TRY(dupload(c, &c.d_fl_dir1, fdir1));
        TRY(dupload(c, &c.d_zar, t0.zar1flux));
        TRY(dupload(c, &c.d_etot, t0.etot));
        TRY(dalloc(c, &c.d_zck, (size_t)c.netot * 2));
        TRY(dalloc(c, &c.d_fpsi, (size_t)std::max<int64_t>(nf, 1) * 4));
        TRY(dalloc(c, &c.d_zcr, (size_t)std::max<int64_t>(nf, 1) * c.netot * 2));
        TRY(dalloc(c, &c.d_zcdr, (size_t)std::max<int64_t>(nf, 1) * c.netot * 2));
        c.d_fring = nullptr;
        c.d_cring = nullptr;
        c.d_zar32 = nullptr;
        if (!c.fp64 && nf > 0) {
            // zeroed: a slot no iteration has written yet adds 0 x 0
            TRY(dalloc(c, &c.d_fring, (size_t)mw3::kFluxSlots * nf * 3));
            TRY(dalloc(c, &c.d_cring, (size_t)mw3::kFluxSlots * c.netot * 2));
            // slices: as many as keep a slice flush at one wave of CTAs or more
            // (2 resident per SM, 64 x 64 tiles), between 4 (a quarter every 32
            // iterations) and kFluxSlots (one slice every iteration)
            const int64_t etiles = (c.netot + 63) / 64;
            int P = 4;
            while (P < mw3::kFluxSlots && ((int64_t)nf / (64 * 2 * P)) * etiles >= 2 * 152) P *= 2;
            c.fl_q = mw3::kFluxSlots / P;
            std::vector<float> zar32(t0.zar1flux.begin(), t0.zar1flux.end());
            TRY(dupload(c, &c.d_zar32, zar32));
        }
        TRY(dalloc(c, &c.d_xj, (size_t)G * n1 * c.nj));
        TRY(dalloc(c, &c.d_cvj, (size_t)G * c.nj * c.nv));
        TRY(dalloc(c, &c.d_zs2, (size_t)G * c.nj * c.nv * c.netot * 2));
        TRY(dupload(c, &c.d_blk_j00, bj00));
        TRY(dupload(c, &c.d_blk_inc, binc));
        TRY(dupload(c, &c.d_blk_isref, bref));
        TRY(dupload(c, &c.d_r2abs, r2abs));
        TRY(dupload(c, &c.d_fd, t0.fd));
        c.d_cvring = c.d_cvcring = c.d_dj32 = c.d_fd32 = c.d_xj32 = nullptr;
        if (!c.fp64) {
            std::vector<float> fd32(t0.fd.begin(), t0.fd.end());
            TRY(dupload(c, &c.d_fd32, fd32));
            // zeroed: a slot no iteration has written yet adds 0 x 0
            TRY(dalloc(c, &c.d_cvring, (size_t)mw3::kFluxRing * G * c.nj * c.nv));
            TRY(dalloc(c, &c.d_cvcring, (size_t)mw3::kFluxRing * c.netot * 2));
            TRY(dalloc(c, &c.d_dj32, (size_t)G * c.nj * na));
            TRY(dalloc(c, &c.d_xj32, (size_t)G * n1 * c.nj));
        }
        TRY(dupload(c, &c.d_nobc, t0.nobc));
    }
    c.wdev.assign(W, WaveDev());
    c.nofemax = 0;
    c.auto_nb = 0;
    for (auto &t : c.waves) c.nofemax = std::max(c.nofemax, t.nofe);
    TRY(dalloc(c, &c.d_zcke, (size_t)W * std::max(c.nofemax, 1) * 2));
    std::vector<double *> zfeptr(W, nullptr), normptr(W, nullptr);
    std::vector<int64_t> normcap(W, 0);
    {
        int64_t foff = 0;
        for (int w = 0; w < W; w++) {
            WaveTables &t = c.waves[w];
            WaveDev &d = c.wdev[w];
            TRY(dupload(c, &d.reacfct, t.reacfct));
            TRY(dupload(c, &d.nelebas, t.nelebas));
            TRY(dupload(c, &d.fl_block, t.fl_block));
            d.zcr = c.d_zcr + (size_t)foff * c.netot * 2;
            d.zcdr = c.d_zcdr + (size_t)foff * c.netot * 2;
            d.zs2 = c.d_zs2 + (size_t)t.g0 * c.nj * c.nv * c.netot * 2;
            d.cvj = c.d_cvj + (size_t)t.g0 * c.nj * c.nv;
            foff += t.nflux;
            d.djmmp = c.d_djall + djoff[w];
            if (t.nofe > 0) {
                TRY(dupload(c, &d.efe, t.efe));
                TRY(dalloc(c, &d.zfe, (size_t)t.nofe * t.ntot * 2));
                zfeptr[w] = d.zfe;
            }
            d.norms_cap = 1024;
            TRY(dalloc(c, &d.norms, (size_t)2 * d.norms_cap));
            if (t.iphoto >= 1) {
                TRY(dalloc(c, &d.psi0, (size_t)t.ntot));
                c.auto_nb = std::max(c.auto_nb, (int)((t.ntot + 2047) / 2048));
            }
            normptr[w] = d.norms;
            normcap[w] = d.norms_cap;
        }
    }
    if (c.auto_nb > 0) TRY(dalloc(c, &c.d_autopart, (size_t)c.auto_nb));
    TRY(dupload(c, &c.d_zfe_ptrs, zfeptr));
    TRY(dupload(c, &c.d_norm_ptrs, normptr));
    TRY(dupload(c, &c.d_norm_cap, normcap));
    // ---- product-state projections (prodpaq / prodcvj) ----
    for (int w = 0; w < W && w < (int)c.prodt.size(); w++) {
        const mw3::ProdTables &pt = c.prodt[w];
        if (!pt.on) continue;
        WaveTables &t = c.waves[w];
        mw3::ProdDev &d = c.wdev[w].prod;
        const int nc = t.ncan, nang = pt.a1 - pt.a0 + 1, n2p = pt.n2p1 - pt.n2p0 + 1;
        std::vector<int> ptr(1, 0);
        std::vector<int64_t> idx;
        std::vector<double> wt;
        std::vector<std::vector<int>> byr2((size_t)n2p);
        for (int b = 0; b < nc; b++)
            for (int iang = pt.a0; iang <= pt.a1; iang++) {
                for (auto &v : byr2) v.clear();
                const int np = c.npunreal[iang - 1];
                for (int ir = 0; ir < np; ir++) {
                    const int ir2 = c.indr2[(size_t)(iang - 1) * c.npt + ir];
                    if (ir2 >= pt.n2p0 && ir2 <= pt.n2p1) byr2[ir2 - pt.n2p0].push_back(ir);
                }
                const int64_t o = t.offs[(size_t)(iang - 1) * nc + b];
                for (int k = 0; k < n2p; k++) {
                    for (int ir : byr2[k]) {
                        idx.push_back(t.flat0 + o + ir);
                        wt.push_back(pt.transrgjac[o + ir]);
                    }
                    ptr.push_back((int)idx.size());
                }
            }
        d.nbins = nc * nang * n2p;
        d.nrow = (pt.om1 - pt.om0 + 1) * (pt.jp1 - pt.jp0 + 1) * (pt.vp1 - pt.vp0 + 1);
        TRY(dupload(c, &d.bin_ptr, ptr));
        TRY(dupload(c, &d.bin_idx, idx));
        TRY(dupload(c, &d.bin_w, wt));
        TRY(dalloc(c, &d.fun, (size_t)d.nbins));
        TRY(dupload(c, &d.dtrans, pt.dtrans));
        TRY(dupload(c, &d.prodwf, pt.prodwf));
        TRY(dupload(c, &d.nobcprod, pt.nobcprod));
        TRY(dupload(c, &d.blk_elec, t.nelebas));
        TRY(dalloc(c, &d.cvjprod, (size_t)d.nrow));
        TRY(dalloc(c, &d.zs2prod, (size_t)d.nrow * c.netot * 2));
    }
    // ---- typed tables ----
    mw3::set_kernel_attributes(c);
    TRY(mw3::build_tc_ang(c));
    TRY(mw3::build_tc_dst2d(c));
    c.h32 = c.use_tc_dst2d && c.use_tc_ang;
    c.d_h32 = nullptr;
    c.d_vr32 = nullptr;
    c.d_pk32 = c.d_pkm1_32 = nullptr;
    if (c.use_tc_dst2d) TRY(dalloc(c, &c.d_h32, (size_t)c.NT));
    if (!c.fp64) {
        // potential pre-scaled for the mixed update: V 2/delta2, minus emindlt 2/delta2 on the diagonal
        const double r2d = 2.0 / c.grid.delta2;
        std::vector<float> vr(c.vvv.size());
        const size_t per = (size_t)c.na * c.npt;
        for (int et = 0; et < c.ne; et++)
            for (int es = 0; es < c.ne; es++) {
                size_t b = ((size_t)et * c.ne + es) * per;
                for (size_t i = 0; i < per; i++)
                    vr[b + i] = (float)(c.vvv[b + i] * r2d - (et == es ? c.grid.emindlt * r2d : 0.0));
            }
        TRY(dupload(c, &c.d_vr32, vr));
        TRY(dalloc(c, &c.d_pk32, c.NT));
        TRY(dalloc(c, &c.d_pkm1_32, c.NT));
    }
    int rc = c.fp64 ? build_typed<double>(c) : build_typed<float>(c);
    if (rc) return rc;
    TRY(alloc_history(c));
    if (c.use_tc_dst2d) TRY(mw3::encode_tc_dst2d_xmap(c));
    if (c.d_dj32) mw3::build_cvj32(c);
    cudaError_t e = cudaStreamSynchronize(c.stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
        c.err = std::string("building device tables: ") + cudaGetErrorString(e);
        return MW3_ERR_CUDA;
    }
    c.built = true;
    c.started = false;
    return MW3_OK;
}

int grow_norms(Ctx &c, int64_t need)
{
    int W = (int)c.waves.size();
    bool changed = false;
    std::vector<double *> ptr(W);
    std::vector<int64_t> cap(W);
    for (int w = 0; w < W; w++) {
        WaveDev &d = c.wdev[w];
        if (need > d.norms_cap) {
            int64_t nc = std::max(need, 2 * d.norms_cap);
            double *p;
            TRY(dalloc(c, &p, (size_t)2 * nc));      // norm trace, then the autocorrelation
            MW3_CUDA_TRY(cudaMemcpyAsync(p, d.norms, sizeof(double) * d.norms_cap, cudaMemcpyDeviceToDevice,
                                         c.stream));
            MW3_CUDA_TRY(cudaMemcpyAsync(p + nc, d.norms + d.norms_cap, sizeof(double) * d.norms_cap,
                                         cudaMemcpyDeviceToDevice, c.stream));
            d.norms = p;
            d.norms_cap = nc;
            changed = true;
        }
        ptr[w] = d.norms;
        cap[w] = d.norms_cap;
    }
    if (changed) {
        MW3_CUDA_TRY(cudaMemcpyAsync(c.d_norm_ptrs, ptr.data(), sizeof(double *) * W, cudaMemcpyHostToDevice,
                                     c.stream));
        MW3_CUDA_TRY(cudaMemcpyAsync(c.d_norm_cap, cap.data(), sizeof(int64_t) * W, cudaMemcpyHostToDevice,
                                     c.stream));
        MW3_CUDA_TRY(cudaStreamSynchronize(c.stream));
    }
    return MW3_OK;
}

template <typename T>
void hphi_typed(Ctx &c, const double *psi, int g0, int g1)
{
    mw3::launch_hphi<T>(c, psi, g0, g1);
}

template <typename T>
void scatter_typed(Ctx &c, const double *psi, int g0, int g1)
{
    // the propagation state also refreshes its FP32 copy (the mixed update reads it)
    mw3::launch_scatter<T>(c, psi, psi == c.d_pk ? c.d_pk32 : nullptr, g0, g1);
}

void scatter(Ctx &c, const double *psi, int g0, int g1)
{
    if (c.fp64) scatter_typed<double>(c, psi, g0, g1);
    else scatter_typed<float>(c, psi, g0, g1);
}

void hphi_all(Ctx &c, const double *psi, int g0, int g1)
{
    if (c.fp64) hphi_typed<double>(c, psi, g0, g1);
    else hphi_typed<float>(c, psi, g0, g1);
}

void update(Ctx &c, int first)
{
    if (c.fp64) mw3::launch_update<double>(c, first);
    else mw3::launch_update<float>(c, first);
}

int check_launch(Ctx &c, const char *where)
{
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        c.err = std::string(where) + ": " + cudaGetErrorString(e);
        return MW3_ERR_CUDA;
    }
    return MW3_OK;
}

// after a synchronisation: did a tensor-core kernel give up waiting for its MMAs?
// The flag is copied in the context's own stream into a pinned word (ordered after
// the context's kernels); a synchronous copy would go through the default stream
// and could wait behind other contexts' transfers on a shared copy engine.
int enqueue_device_flags(Ctx &c)
{
    if (!c.d_tc_err || !c.h_flag) return MW3_OK;
    MW3_CUDA_TRY(cudaMemcpyAsync(c.h_flag, c.d_tc_err, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    return MW3_OK;
}

// after enqueue_device_flags and a synchronisation of the context's stream
int device_flags_result(Ctx &c, const char *where)
{
    if (!c.d_tc_err || !c.h_flag || !*c.h_flag) return MW3_OK;
    c.err = std::string(where) + ": a tensor-core kernel timed out waiting for its MMAs";
    return MW3_ERR_CUDA;
}

int check_device_flags(Ctx &c, const char *where)
{
    int rc = enqueue_device_flags(c);
    if (rc) return rc;
    MW3_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return device_flags_result(c, where);
}

int reset_accumulators(Ctx &c)
{
    size_t nf = (size_t)std::max(c.NF, 1) * c.netot * 2;
    if (c.d_cvcring)
        MW3_CUDA_TRY(cudaMemsetAsync(c.d_cvcring, 0, sizeof(float) * mw3::kFluxRing * c.netot * 2, c.stream));
    if (c.d_cring)
        MW3_CUDA_TRY(cudaMemsetAsync(c.d_cring, 0, sizeof(float) * mw3::kFluxSlots * c.netot * 2, c.stream));
    MW3_CUDA_TRY(cudaMemsetAsync(c.d_zcr, 0, sizeof(double) * nf, c.stream));
    MW3_CUDA_TRY(cudaMemsetAsync(c.d_zcdr, 0, sizeof(double) * nf, c.stream));
    MW3_CUDA_TRY(cudaMemsetAsync(c.d_zs2, 0, sizeof(double) * 2 * (size_t)c.G * c.nj * c.nv * c.netot, c.stream));
    MW3_CUDA_TRY(cudaMemsetAsync(c.d_cvj, 0, sizeof(double) * (size_t)c.G * c.nj * c.nv, c.stream));
    for (size_t w = 0; w < c.waves.size(); w++) {
        WaveTables &t = c.waves[w];
        WaveDev &d = c.wdev[w];
        if (d.zfe) MW3_CUDA_TRY(cudaMemsetAsync(d.zfe, 0, sizeof(double) * 2 * (size_t)t.nofe * t.ntot, c.stream));
        if (d.prod.zs2prod) {
            MW3_CUDA_TRY(cudaMemsetAsync(d.prod.zs2prod, 0, sizeof(double) * 2 * (size_t)d.prod.nrow * c.netot,
                                         c.stream));
            MW3_CUDA_TRY(cudaMemsetAsync(d.prod.cvjprod, 0, sizeof(double) * (size_t)d.prod.nrow, c.stream));
        }
    }
    return MW3_OK;
}

}  // namespace

namespace mw3 {
void stage_mark(Ctx &c, int stage)
{
    if (!c.prof || c.prof_n >= c.prof_cap) return;
    cudaEventRecord(c.prof_ev[(size_t)c.prof_n * (MW3_NSTAGES + 1) + stage], c.stream);
}
int api_check_launch(Ctx &c, const char *where) { return check_launch(c, where); }
int api_check_device_flags(Ctx &c, const char *where) { return check_device_flags(c, where); }
}  // namespace mw3

static int start_device(Ctx &c);

// ===========================================================================
// C-ABI
// ===========================================================================
extern "C" {

int mw3_create(mw3_ctx **out, const mw3_grid *g, const int32_t *npunreal, const int32_t *indr1,
               const int32_t *indr2, const double *vvv)
{
    if (!out || !g || !npunreal || !indr1 || !indr2 || !vvv) return MW3_ERR_ARG;
    *out = nullptr;
    if (g->npun1 < 2 || g->npun2 < 2 || g->nangu < 1 || g->nelec < 1 || g->nelec > 8 || g->npuntot < 1 ||
        g->npun1 > 256 || g->nangu > 2047 || g->npuntot >= (1 << 20) ||
        (g->precision != MW3_PREC_FP64 && g->precision != MW3_PREC_MIXED))
        return MW3_ERR_ARG;
    if (!(g->delta2 > 0.0) || !(g->rfin1 > g->rmis1) || !(g->rfin2 > g->rmis2)) return MW3_ERR_ARG;
    mw3_ctx *h = new (std::nothrow) mw3_ctx();
    if (!h) return MW3_ERR_NOMEM;
    Ctx &c = h->c;
    c.grid = *g;
    c.n1 = g->npun1;
    c.n2 = g->npun2;
    c.na = g->nangu;
    c.ne = g->nelec;
    c.npt = g->npuntot;
    c.fp64 = (g->precision == MW3_PREC_FP64);
    const char *ng = std::getenv("MW3_NO_GRAPHS");
    c.graphs_off = ng && ng[0] == '1';
    c.npunreal.assign(npunreal, npunreal + c.na);
    c.indr1.assign(indr1, indr1 + (size_t)c.na * c.npt);
    c.indr2.assign(indr2, indr2 + (size_t)c.na * c.npt);
    c.vvv.assign(vvv, vvv + (size_t)c.ne * c.ne * c.na * c.npt);
    for (int a = 0; a < c.na; a++) {
        if (c.npunreal[a] < 1 || c.npunreal[a] > c.npt) {
            delete h;
            return MW3_ERR_ARG;
        }
        for (int ir = 0; ir < c.npunreal[a]; ir++) {
            int r1 = c.indr1[(size_t)a * c.npt + ir], r2 = c.indr2[(size_t)a * c.npt + ir];
            if (r1 < 1 || r1 > c.n1 || r2 < 1 || r2 > c.n2) {
                delete h;
                return MW3_ERR_ARG;
            }
        }
    }
    cudaError_t e = cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) {
        e = cudaHostAlloc((void **)&c.h_flag, sizeof(int), cudaHostAllocDefault);
        if (e == cudaSuccess) *c.h_flag = 0;
        else cudaStreamDestroy(c.stream);
    }
    if (e != cudaSuccess) {
        delete h;
        return MW3_ERR_CUDA;
    }
    int dev = 0;
    cudaDeviceProp prop;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaGetDeviceProperties(&prop, dev) == cudaSuccess) {
        // the dynamic shared memory the kernels need must fit the device (the
        // explicit angular kernels narrow their column chunk for large angle counts)
        if (!mw3::fit_smem(c, prop.sharedMemPerBlockOptin)) {
            cudaStreamDestroy(c.stream);
            cudaFreeHost(c.h_flag);
            delete h;
            return MW3_ERR_UNSUPPORTED;
        }
    }
    c.ang_cw_fit = c.ang_cw;
    *out = h;
    return MW3_OK;
}

int mw3_add_wave(mw3_ctx *h, const mw3_wave *w, int32_t *wave_id)
{
    if (!h || !w) return MW3_ERR_ARG;
    Ctx &c = h->c;
    if (!w->iombas || !w->nelebas || !w->nojbas || !w->j00 || !w->jbas || !w->iomdiat || !w->iomatom ||
        !w->sigdiat || !w->sigatom || !w->djmmp || !w->nobc || !w->ediat || !w->fd || (w->nofe > 0 && !w->efe)) {
        c.err = "mw3_add_wave: null array";
        return MW3_ERR_ARG;
    }
    WaveTables t;
    std::string err;
    int rc = mw3::build_wave_tables(c, *w, t, err);
    if (rc) {
        c.err = "mw3_add_wave: " + err;
        return rc;
    }
    c.waves.push_back(std::move(t));
    c.built = false;
    c.started = false;
    if (wave_id) *wave_id = (int32_t)c.waves.size() - 1;
    return MW3_OK;
}

int mw3_wave_size(mw3_ctx *h, int32_t w, int64_t *ntot)
{
    if (!h || !ntot || w < 0 || w >= (int)h->c.waves.size()) return MW3_ERR_ARG;
    *ntot = h->c.waves[w].ntot;
    return MW3_OK;
}

int mw3_hphi(mw3_ctx *h, int32_t w, const double *psi, double *hpsi)
{
    if (!h || !psi || !hpsi) return MW3_ERR_ARG;
    Ctx &c = h->c;
    if (w < 0 || w >= (int)c.waves.size()) return MW3_ERR_ARG;
    int rc = build_device(c);
    if (rc) return rc;
    WaveTables &t = c.waves[w];
    MW3_CUDA_TRY(cudaMemcpyAsync(c.d_tmp + t.flat0, psi, sizeof(double) * t.ntot, cudaMemcpyHostToDevice, c.stream));
    scatter(c, c.d_tmp, t.g0, t.g0 + t.ncan);
    hphi_all(c, c.d_tmp, t.g0, t.g0 + t.ncan);
    // V psi (the update kernel adds it during propagation)
    mw3::launch_addv(c, c.d_tmp, t.g0, t.g0 + t.ncan);
    MW3_CUDA_TRY(cudaMemcpyAsync(hpsi, c.d_h + t.flat0, sizeof(double) * t.ntot, cudaMemcpyDeviceToHost, c.stream));
    if (c.started) scatter(c, c.d_pk, t.g0, t.g0 + t.ncan);   // restore the propagation rectangle
    rc = check_launch(c, "mw3_hphi");
    if (rc) return rc;
    MW3_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return check_device_flags(c, "mw3_hphi");
}

int mw3_start(mw3_ctx *h, const double *const *psi0s)
{
    if (!h || !psi0s) return MW3_ERR_ARG;
    Ctx &c = h->c;
    int rc = build_device(c);
    if (rc) return rc;
    for (size_t w = 0; w < c.waves.size(); w++) {
        WaveTables &t = c.waves[w];
        if (!psi0s[w]) return MW3_ERR_ARG;
        MW3_CUDA_TRY(cudaMemcpyAsync(c.d_pk + t.flat0, psi0s[w], sizeof(double) * t.ntot, cudaMemcpyHostToDevice,
                                     c.stream));
    }
    return start_device(c);
}
}  // extern "C"

// the first Chebyshev step from the packets already in c.d_pk (main_madwave3.f:238-250)
static int start_device(Ctx &c)
{
    int rc;
    MW3_CUDA_TRY(cudaMemcpyAsync(c.d_pkm1, c.d_pk, sizeof(double) * c.NT, cudaMemcpyDeviceToDevice, c.stream));
    for (size_t w = 0; w < c.waves.size(); w++)   // check's rpaq0 of the photodissociation waves
        if (c.wdev[w].psi0)
            MW3_CUDA_TRY(cudaMemcpyAsync(c.wdev[w].psi0, c.d_pk + c.waves[w].flat0, sizeof(double) * c.waves[w].ntot,
                                         cudaMemcpyDeviceToDevice, c.stream));
    rc = reset_accumulators(c);
    if (rc) return rc;
    scatter(c, c.d_pk, 0, c.G);
    hphi_all(c, c.d_pk, 0, c.G);
    update(c, 1);
    std::swap(c.d_pk, c.d_pkm1);
    std::swap(c.d_pk32, c.d_pkm1_32);
    mw3::launch_norms(c, 0);
    if (c.auto_nb > 0) mw3::launch_autocorr(c, 0);
    c.it = 1;
    c.norm_slot = 1;
    c.hist_n = 0;
    c.started = true;
    return check_launch(c, "mw3_start");
}

extern "C" {

int mw3_upload_state(mw3_ctx *h, int32_t w, const double *psi_km1, const double *psi_k, int64_t it)
{
    if (!h || !psi_km1 || !psi_k || it < 1) return MW3_ERR_ARG;
    Ctx &c = h->c;
    if (w < 0 || w >= (int)c.waves.size()) return MW3_ERR_ARG;
    int rc = build_device(c);
    if (rc) return rc;
    if (c.started && it != c.it && c.waves.size() > 1) {
        c.err = "all partial waves of a context share the iteration index";
        return MW3_ERR_STATE;
    }
    WaveTables &t = c.waves[w];
    MW3_CUDA_TRY(cudaMemcpyAsync(c.d_pkm1 + t.flat0, psi_km1, sizeof(double) * t.ntot, cudaMemcpyHostToDevice,
                                 c.stream));
    MW3_CUDA_TRY(cudaMemcpyAsync(c.d_pk + t.flat0, psi_k, sizeof(double) * t.ntot, cudaMemcpyHostToDevice,
                                 c.stream));
    scatter(c, c.d_pk, t.g0, t.g0 + t.ncan);
    if (!c.started) {
        rc = reset_accumulators(c);
        if (rc) return rc;
    }
    if (c.started && it != c.it) {   // the rings' slots follow the iteration
        mw3::flush_flux(c);
        mw3::flush_cvj(c);
    }
    c.it = it;
    c.norm_slot = 0;
    c.hist_n = 0;
    c.started = true;
    rc = check_launch(c, "mw3_upload_state");
    if (rc) return rc;
    MW3_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return MW3_OK;
}

}  // extern "C"

namespace {

// one Chebyshev iteration of every wave, launched on the context's stream
void run_iteration(Ctx &c)
{
    int64_t it = c.it + 1;
    hphi_all(c, c.d_pk, 0, c.G);
    if (c.nofemax > 0) mw3::launch_fe_coef(c, it);
    update(c, 0);
    std::swap(c.d_pk, c.d_pkm1);
    std::swap(c.d_pk32, c.d_pkm1_32);
    mw3::launch_accumulators(c, it);
    mw3::launch_norms(c, c.norm_slot);
    if (c.auto_nb > 0) mw3::launch_autocorr(c, c.norm_slot);
    mw3::launch_cvj_keep(c, it, c.norm_slot);
    if (c.hist_cap > 0) c.hist_n = std::min(c.hist_n + 1, c.hist_cap);
    if (c.prof && c.prof_n < c.prof_cap) {
        mw3::stage_mark(c, MW3_NSTAGES);
        c.prof_n++;
    }
    c.it = it;
    c.norm_slot++;
}

// a block of kGraphIters iterations repeats exactly when it starts at an iteration
// that is a multiple of kGraphIters (the rings' slots and flushes follow the
// iteration number modulo 32, or, for the flux ring's slots, a replay reads it on
// the device), no iteration of the block is gated (the elastic channel below
// kminelastic changes the launches) and no stage timing is recorded
bool graph_ready(Ctx &c, int64_t left)
{
    if (c.graphs_off || c.prof || left < mw3::kGraphIters) return false;
    if (c.it % mw3::kGraphIters != 0) return false;
    if (c.gate_elastic && c.it + 1 < c.kminelastic) return false;
    return true;
}

// capture kGraphIters iterations starting from the current psi buffer parity; the
// host-side state the eager launches advance is put back afterwards
void capture_graph(Ctx &c, int par)
{
    if (!c.d_itbase) {
        if (cudaMalloc((void **)&c.d_itbase, 2 * sizeof(int64_t)) != cudaSuccess) {
            c.graphs_off = true;
            return;
        }
        c.allocs.push_back(c.d_itbase);
    }
    const int64_t it0 = c.it, slot0 = c.norm_slot, l0 = c.launches, h0 = c.hist_n;
    double *pk = c.d_pk, *pkm1 = c.d_pkm1;
    float *pk32 = c.d_pk32, *pkm1_32 = c.d_pkm1_32;
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        c.graphs_off = true;
        return;
    }
    c.capturing = true;
    c.cap_it0 = it0;
    c.cap_slot0 = slot0;
    for (int i = 0; i < mw3::kGraphIters; i++) run_iteration(c);
    c.capturing = false;
    cudaError_t e = cudaStreamEndCapture(c.stream, &g);
    const int64_t launches = c.launches - l0;
    c.it = it0;
    c.norm_slot = slot0;
    c.hist_n = h0;
    c.d_pk = pk;
    c.d_pkm1 = pkm1;
    c.d_pk32 = pk32;
    c.d_pkm1_32 = pkm1_32;
    c.launches = l0;
    if (e == cudaSuccess && g && cudaGraphInstantiate(&c.graph_exec[par], g, 0) == cudaSuccess) {
        c.graph_launches[par] = launches;
    } else {
        c.graph_exec[par] = nullptr;
        c.graphs_off = true;
        cudaGetLastError();
    }
    if (g) cudaGraphDestroy(g);
}

}  // namespace

extern "C" {

int mw3_run(mw3_ctx *h, int64_t n)
{
    if (!h || n < 0) return MW3_ERR_ARG;
    Ctx &c = h->c;
    if (!c.started) {
        c.err = "mw3_run before mw3_start/mw3_upload_state";
        return MW3_ERR_STATE;
    }
    int rc = grow_norms(c, c.norm_slot + n);
    if (rc) return rc;
    if (c.prof && c.prof_n + n > c.prof_cap) {
        int64_t need = c.prof_n + n;
        size_t old = c.prof_ev.size();
        c.prof_ev.resize((size_t)need * (MW3_NSTAGES + 1));
        for (size_t i = old; i < c.prof_ev.size(); i++) MW3_CUDA_TRY(cudaEventCreate(&c.prof_ev[i]));
        c.prof_cap = need;
    }
    for (int64_t s = 0; s < n;) {
        if (graph_ready(c, n - s)) {
            // kGraphIters iterations as one graph replay
            const int par = c.d_pk == c.d_psiA ? 0 : 1;
            if (!c.graph_exec[par]) capture_graph(c, par);
            if (c.graph_exec[par]) {
                mw3::launch_set_itbase(c);
                MW3_CUDA_TRY(cudaGraphLaunch(c.graph_exec[par], c.stream));
                c.launches += c.graph_launches[par];
                c.it += mw3::kGraphIters;
                c.norm_slot += mw3::kGraphIters;
                if (c.hist_cap > 0) c.hist_n = std::min(c.hist_n + mw3::kGraphIters, c.hist_cap);
                s += mw3::kGraphIters;
                continue;
            }
        }
        run_iteration(c);
        s++;
    }
    return check_launch(c, "mw3_run");
}

int mw3_sync(mw3_ctx *h)
{
    if (!h) return MW3_ERR_ARG;
    Ctx &c = h->c;
    MW3_CUDA_TRY(cudaStreamSynchronize(c.stream));
    int rc = check_launch(c, "mw3_sync");
    if (rc) return rc;
    return check_device_flags(c, "mw3_sync");
}

int mw3_download_state(mw3_ctx *h, int32_t w, double *km1, double *k, int64_t *it)
{
    if (!h) return MW3_ERR_ARG;
    Ctx &c = h->c;
    if (w < 0 || w >= (int)c.waves.size() || !c.started) return MW3_ERR_STATE;
    WaveTables &t = c.waves[w];
    if (km1)
        MW3_CUDA_TRY(cudaMemcpyAsync(km1, c.d_pkm1 + t.flat0, sizeof(double) * t.ntot, cudaMemcpyDeviceToHost,
                                     c.stream));
    if (k)
        MW3_CUDA_TRY(cudaMemcpyAsync(k, c.d_pk + t.flat0, sizeof(double) * t.ntot, cudaMemcpyDeviceToHost,
                                     c.stream));
    MW3_CUDA_TRY(cudaStreamSynchronize(c.stream));
    if (it) *it = c.it;
    return check_device_flags(c, "mw3_download_state");
}

int mw3_upload_state_all(mw3_ctx *h, const double *psi_km1, const double *psi_k, int64_t it)
{
    if (!h || !psi_k || it < 1) return MW3_ERR_ARG;
    Ctx &c = h->c;
    if (!psi_km1 && !c.started) {
        c.err = "mw3_upload_state_all: psi_km1 may be NULL only once the context holds a state";
        return MW3_ERR_STATE;
    }
    int rc = build_device(c);
    if (rc) return rc;
    if (psi_km1)
        MW3_CUDA_TRY(cudaMemcpyAsync(c.d_pkm1, psi_km1, sizeof(double) * c.NT, cudaMemcpyHostToDevice, c.stream));
    MW3_CUDA_TRY(cudaMemcpyAsync(c.d_pk, psi_k, sizeof(double) * c.NT, cudaMemcpyHostToDevice, c.stream));
    scatter(c, c.d_pk, 0, c.G);
    if (!c.started) {
        rc = reset_accumulators(c);
        if (rc) return rc;
    }
    if (c.started && it != c.it) {   // the rings' slots follow the iteration
        mw3::flush_flux(c);
        mw3::flush_cvj(c);
    }
    c.it = it;
    c.norm_slot = 0;
    c.hist_n = 0;
    c.started = true;
    rc = check_launch(c, "mw3_upload_state_all");
    if (rc) return rc;
    MW3_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return MW3_OK;
}

int mw3_download_state_all(mw3_ctx *h, double *km1, double *k, int64_t *it)
{
    if (!h) return MW3_ERR_ARG;
    Ctx &c = h->c;
    if (!c.started) return MW3_ERR_STATE;
    if (km1) MW3_CUDA_TRY(cudaMemcpyAsync(km1, c.d_pkm1, sizeof(double) * c.NT, cudaMemcpyDeviceToHost, c.stream));
    if (k) MW3_CUDA_TRY(cudaMemcpyAsync(k, c.d_pk, sizeof(double) * c.NT, cudaMemcpyDeviceToHost, c.stream));
    int rc = enqueue_device_flags(c);
    if (rc) return rc;
    MW3_CUDA_TRY(cudaStreamSynchronize(c.stream));
    if (it) *it = c.it;
    return device_flags_result(c, "mw3_download_state_all");
}

int mw3_norms(mw3_ctx *h, int32_t w, double *norms, int64_t *n)
{
    if (!h || !n) return MW3_ERR_ARG;
    Ctx &c = h->c;
    if (w < 0 || w >= (int)c.waves.size() || !c.started) return MW3_ERR_STATE;
    int64_t m = std::min(*n, c.norm_slot);
    if (norms && m > 0)
        MW3_CUDA_TRY(cudaMemcpyAsync(norms, c.wdev[w].norms, sizeof(double) * m, cudaMemcpyDeviceToHost, c.stream));
    MW3_CUDA_TRY(cudaStreamSynchronize(c.stream));
    *n = m;
    return MW3_OK;
}

int mw3_autocorrelation(mw3_ctx *h, int32_t w, double *autos, int64_t *n)
{
    if (!h || !n) return MW3_ERR_ARG;
    Ctx &c = h->c;
    if (w < 0 || w >= (int)c.waves.size() || !c.started) return MW3_ERR_STATE;
    if (!c.wdev[w].psi0) {
        c.err = "mw3_autocorrelation: the wave is not a photodissociation (iphoto >= 1)";
        return MW3_ERR_STATE;
    }
    int64_t m = std::min(*n, c.norm_slot);
    if (autos && m > 0)
        MW3_CUDA_TRY(cudaMemcpyAsync(autos, c.wdev[w].norms + c.wdev[w].norms_cap, sizeof(double) * m,
                                     cudaMemcpyDeviceToHost, c.stream));
    MW3_CUDA_TRY(cudaStreamSynchronize(c.stream));
    *n = m;
    return check_device_flags(c, "mw3_autocorrelation");
}

int mw3_totalflux(mw3_ctx *h, int32_t w, double *tot, double *elec)
{
    if (!h || !tot) return MW3_ERR_ARG;
    Ctx &c = h->c;
    if (w < 0 || w >= (int)c.waves.size() || !c.built) return MW3_ERR_STATE;
    WaveTables &t = c.waves[w];
    double *d = nullptr;
    mw3::flush_flux(c);
    mw3::flush_cvj(c);
    MW3_CUDA_TRY(cudaMallocAsync(&d, sizeof(double) * (size_t)t.netot * (1 + c.ne), c.stream));
    mw3::launch_totalflux(c, w, d, d + t.netot);
    MW3_CUDA_TRY(cudaMemcpyAsync(tot, d, sizeof(double) * t.netot, cudaMemcpyDeviceToHost, c.stream));
    if (elec)
        MW3_CUDA_TRY(cudaMemcpyAsync(elec, d + t.netot, sizeof(double) * (size_t)t.netot * c.ne,
                                     cudaMemcpyDeviceToHost, c.stream));
    MW3_CUDA_TRY(cudaFreeAsync(d, c.stream));
    MW3_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return check_launch(c, "mw3_totalflux");
}

int mw3_flux_count(mw3_ctx *h, int32_t w, int32_t *nflux)
{
    if (!h || !nflux || w < 0 || w >= (int)h->c.waves.size()) return MW3_ERR_ARG;
    *nflux = h->c.waves[w].nflux;
    return MW3_OK;
}

int mw3_download_accumulators(mw3_ctx *h, int32_t w, double *zcr, double *zcdr, double *zs2, double *cvj,
                              double *zfe)
{
    if (!h) return MW3_ERR_ARG;
    Ctx &c = h->c;
    if (w < 0 || w >= (int)c.waves.size() || !c.built) return MW3_ERR_STATE;
    WaveTables &t = c.waves[w];
    WaveDev &d = c.wdev[w];
    size_t nf = (size_t)t.nflux * t.netot * 2;
    size_t ns = (size_t)t.ncan * t.nj * t.nv;
    mw3::flush_flux(c);
    mw3::flush_cvj(c);
    if (zcr && nf) MW3_CUDA_TRY(cudaMemcpyAsync(zcr, d.zcr, sizeof(double) * nf, cudaMemcpyDeviceToHost, c.stream));
    if (zcdr && nf)
        MW3_CUDA_TRY(cudaMemcpyAsync(zcdr, d.zcdr, sizeof(double) * nf, cudaMemcpyDeviceToHost, c.stream));
    if (zs2)
        MW3_CUDA_TRY(cudaMemcpyAsync(zs2, d.zs2, sizeof(double) * ns * t.netot * 2, cudaMemcpyDeviceToHost, c.stream));
    if (cvj) MW3_CUDA_TRY(cudaMemcpyAsync(cvj, d.cvj, sizeof(double) * ns, cudaMemcpyDeviceToHost, c.stream));
    if (zfe && d.zfe)
        MW3_CUDA_TRY(cudaMemcpyAsync(zfe, d.zfe, sizeof(double) * 2 * (size_t)t.nofe * t.ntot, cudaMemcpyDeviceToHost,
                                     c.stream));
    MW3_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return MW3_OK;
}

int mw3_upload_accumulators(mw3_ctx *h, int32_t w, const double *zcr, const double *zcdr, const double *zs2)
{
    if (!h) return MW3_ERR_ARG;
    Ctx &c = h->c;
    if (w < 0 || w >= (int)c.waves.size()) return MW3_ERR_ARG;
    if (!c.built || !c.started) {
        c.err = "mw3_upload_accumulators: upload the state first";
        return MW3_ERR_STATE;
    }
    WaveTables &t = c.waves[w];
    WaveDev &d = c.wdev[w];
    size_t nf = (size_t)t.nflux * t.netot * 2;
    size_t ns = (size_t)t.ncan * t.nj * t.nv;
    mw3::flush_flux(c);
    mw3::flush_cvj(c);
    if (zcr && nf) MW3_CUDA_TRY(cudaMemcpyAsync(d.zcr, zcr, sizeof(double) * nf, cudaMemcpyHostToDevice, c.stream));
    if (zcdr && nf)
        MW3_CUDA_TRY(cudaMemcpyAsync(d.zcdr, zcdr, sizeof(double) * nf, cudaMemcpyHostToDevice, c.stream));
    if (zs2)
        MW3_CUDA_TRY(cudaMemcpyAsync(d.zs2, zs2, sizeof(double) * ns * t.netot * 2, cudaMemcpyHostToDevice, c.stream));
    MW3_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return check_launch(c, "mw3_upload_accumulators");
}

int mw3_tables(mw3_ctx *h, int32_t w, int32_t *nopr1, double *etot, double *reacfct, double *s2factor,
               double *absfr1, double *absfr2)
{
    if (!h || w < 0 || w >= (int)h->c.waves.size()) return MW3_ERR_ARG;
    WaveTables &t = h->c.waves[w];
    if (nopr1) std::copy(t.nopr1.begin(), t.nopr1.end(), nopr1);
    if (etot) std::copy(t.etot.begin(), t.etot.end(), etot);
    if (reacfct) std::copy(t.reacfct.begin(), t.reacfct.end(), reacfct);
    if (s2factor) std::copy(t.s2factor.begin(), t.s2factor.end(), s2factor);
    if (absfr1) std::copy(t.absfr1.begin(), t.absfr1.end(), absfr1);
    if (absfr2) std::copy(t.absfr2.begin(), t.absfr2.end(), absfr2);
    return MW3_OK;
}

int mw3_set_ecoriolis(mw3_ctx *h, int32_t w, int32_t on)
{
    if (!h) return MW3_ERR_ARG;
    Ctx &c = h->c;
    if (w < 0 || w >= (int)c.waves.size()) {
        c.err = "mw3_set_ecoriolis: no such wave";
        return MW3_ERR_ARG;
    }
    if (c.built) {
        c.err = "mw3_set_ecoriolis: call before the device tables exist";
        return MW3_ERR_STATE;
    }
    c.waves[w].ecor = on != 0;
    return MW3_OK;
}

int mw3_set_flux_gate(mw3_ctx *h, int32_t w, int32_t on)
{
    if (!h || w < 0 || w >= (int)h->c.waves.size()) return MW3_ERR_ARG;
    Ctx &c = h->c;
    if (c.built) {
        c.err = "mw3_set_flux_gate: call before the device tables exist";
        return MW3_ERR_STATE;
    }
    c.waves[w].flux_gate = on != 0;
    return MW3_OK;
}

int mw3_packet_energy_norm(mw3_ctx *h, int32_t w, double *apaqini)
{
    if (!h || !apaqini || w < 0 || w >= (int)h->c.waves.size()) return MW3_ERR_ARG;
    const WaveTables &t = h->c.waves[w];
    std::copy(t.apaqini.begin(), t.apaqini.end(), apaqini);
    return MW3_OK;
}

int mw3_cvj_history(mw3_ctx *h, int64_t capacity)
{
    if (!h || capacity < 0) return MW3_ERR_ARG;
    Ctx &c = h->c;
    for (int p = 0; p < 2; p++) {   // captured blocks must include (or drop) the record
        if (c.graph_exec[p]) cudaGraphExecDestroy(c.graph_exec[p]);
        c.graph_exec[p] = nullptr;
        c.graph_launches[p] = 0;
    }
    c.hist_cap = capacity;
    if (!c.built) return MW3_OK;
    MW3_CUDA_TRY(cudaStreamSynchronize(c.stream));
    int rc = alloc_history(c);
    if (rc) return rc;
    return check_launch(c, "mw3_cvj_history");
}

int mw3_download_cvj_history(mw3_ctx *h, int32_t w, int64_t n, double *cvj, double *cvjprod, int64_t *it_last)
{
    if (!h || n < 0) return MW3_ERR_ARG;
    Ctx &c = h->c;
    if (w < 0 || w >= (int)c.waves.size()) return MW3_ERR_ARG;
    if (!c.built || c.hist_cap <= 0) {
        c.err = "mw3_download_cvj_history: no history enabled (mw3_cvj_history)";
        return MW3_ERR_STATE;
    }
    if (n > c.hist_n) {
        c.err = "mw3_download_cvj_history: " + std::to_string(n) + " iterations asked, " +
                std::to_string(c.hist_n) + " recorded";
        return MW3_ERR_ARG;
    }
    const WaveTables &t = c.waves[w];
    const mw3::ProdDev &d = c.wdev[w].prod;
    if (cvjprod && !d.cvjph) {
        c.err = "mw3_download_cvj_history: the wave has no product projection";
        return MW3_ERR_ARG;
    }
    const size_t R = (size_t)c.G * c.nj * c.nv, per = (size_t)t.ncan * c.nj * c.nv;
    for (int64_t k = 0; k < n; k++) {
        const int64_t slot = ((c.norm_slot - n + k) % c.hist_cap + c.hist_cap) % c.hist_cap;
        if (cvj && c.d_cvjh)
            MW3_CUDA_TRY(cudaMemcpyAsync(cvj + (size_t)k * per, c.d_cvjh + (size_t)slot * R + (size_t)t.g0 * c.nj * c.nv,
                                         sizeof(double) * per, cudaMemcpyDeviceToHost, c.stream));
        if (cvjprod)
            MW3_CUDA_TRY(cudaMemcpyAsync(cvjprod + (size_t)k * d.nrow, d.cvjph + (size_t)slot * d.nrow,
                                         sizeof(double) * d.nrow, cudaMemcpyDeviceToHost, c.stream));
    }
    MW3_CUDA_TRY(cudaStreamSynchronize(c.stream));
    if (it_last) *it_last = c.it;
    return check_device_flags(c, "mw3_download_cvj_history");
}

int mw3_kernel_launches(mw3_ctx *h, int64_t *count)
{
    if (!h || !count) return MW3_ERR_ARG;
    *count = h->c.launches;
    return MW3_OK;
}

int mw3_path_flags(mw3_ctx *h, int32_t *flags)
{
    if (!h || !flags) return MW3_ERR_ARG;
    Ctx &c = h->c;
    if (!c.built) {
        c.err = "mw3_path_flags before the device tables were built";
        return MW3_ERR_STATE;
    }
    *flags = ((mw3::tc_dst_supported(c) || c.use_tc_dst2d) ? MW3_PATH_TC_DST : 0) |
             (c.use_tc_dst2d ? MW3_PATH_TC_DST_FUSED : 0) | (c.use_tc_ang ? MW3_PATH_TC_ANG : 0) |
             ((c.use_tc_dst2d && c.dst_f16) ? MW3_PATH_DST_F16 : 0) | (c.x_t ? MW3_PATH_X_T : 0) |
             ((c.fp64 && c.d_rd_tw) ? MW3_PATH_RADER : 0);
    return MW3_OK;
}

int mw3_get_stream(mw3_ctx *h, void **stream)
{
    if (!h || !stream) return MW3_ERR_ARG;
    *stream = (void *)h->c.stream;
    return MW3_OK;
}

int mw3_profile(mw3_ctx *h, int enable)
{
    if (!h) return MW3_ERR_ARG;
    h->c.prof = enable != 0;
    h->c.prof_n = 0;
    return MW3_OK;
}

int mw3_stage_times(mw3_ctx *h, double *ms, int64_t *iterations)
{
    if (!h || !ms) return MW3_ERR_ARG;
    Ctx &c = h->c;
    MW3_CUDA_TRY(cudaStreamSynchronize(c.stream));
    for (int s = 0; s < MW3_NSTAGES; s++) ms[s] = 0.0;
    for (int64_t i = 0; i < c.prof_n; i++) {
        cudaEvent_t *e = &c.prof_ev[(size_t)i * (MW3_NSTAGES + 1)];
        // stages without their own start mark (no angular kernels) fold into the next one
        for (int s = 0; s < MW3_NSTAGES; s++) {
            float t = 0.f;
            if (cudaEventElapsedTime(&t, e[s], e[s + 1]) == cudaSuccess) ms[s] += t;
        }
    }
    cudaGetLastError();
    if (iterations) *iterations = c.prof_n;
    c.prof_n = 0;
    return MW3_OK;
}

int mw3_set_product_projection(mw3_ctx *h, int32_t w, const mw3_prodproj *p)
{
    if (!h || !p) return MW3_ERR_ARG;
    Ctx &c = h->c;
    if (w < 0 || w >= (int)c.waves.size()) return MW3_ERR_ARG;
    if (c.built) {
        c.err = "mw3_set_product_projection: set it before the device tables are built";
        return MW3_ERR_STATE;
    }
    if (!p->nobcprod || !p->transrgjac || !p->dtrans || !p->prodwf) return MW3_ERR_ARG;
    if (p->n2prod0 < 1 || p->n2prod1 < p->n2prod0 || p->n2prod1 > c.n2 || p->nangproj0 < 1 ||
        p->nangproj1 < p->nangproj0 || p->nangproj1 > c.na || p->iommaxprod < p->iomminprod ||
        p->jmaxprod < p->jiniprod || p->nvmaxprod < p->nviniprod || p->iomminprod < 0)
        return MW3_ERR_ARG;
    const WaveTables &t = c.waves[w];
    const size_t n2p = p->n2prod1 - p->n2prod0 + 1, nang = p->nangproj1 - p->nangproj0 + 1;
    const size_t nom = p->iommaxprod - p->iomminprod + 1, njp = p->jmaxprod - p->jiniprod + 1;
    const size_t nvp = p->nvmaxprod - p->nviniprod + 1;
    if ((double)nom * njp * nvp * c.netot > 2.0e9 || (double)t.ncan * nang * n2p > 2.0e9) return MW3_ERR_ARG;
    for (size_t j = 0; j < njp; j++)
        if (p->nobcprod[j] > p->nvmaxprod) return MW3_ERR_ARG;
    if (c.prodt.size() < c.waves.size()) c.prodt.resize(c.waves.size());
    mw3::ProdTables &pt = c.prodt[w];
    pt.on = true;
    pt.n2p0 = p->n2prod0; pt.n2p1 = p->n2prod1; pt.a0 = p->nangproj0; pt.a1 = p->nangproj1;
    pt.om0 = p->iomminprod; pt.om1 = p->iommaxprod; pt.jp0 = p->jiniprod; pt.jp1 = p->jmaxprod;
    pt.vp0 = p->nviniprod; pt.vp1 = p->nvmaxprod;
    pt.nobcprod.assign(p->nobcprod, p->nobcprod + njp);
    pt.transrgjac.assign(p->transrgjac, p->transrgjac + t.ntot);
    pt.dtrans.assign(p->dtrans, p->dtrans + (size_t)t.ncan * nom * nang * n2p);
    pt.prodwf.assign(p->prodwf, p->prodwf + nom * njp * nvp * (size_t)c.ne * nang * n2p);
    return MW3_OK;
}

int mw3_download_product(mw3_ctx *h, int32_t w, double *zs2prod, double *cvjprod)
{
    if (!h) return MW3_ERR_ARG;
    Ctx &c = h->c;
    if (w < 0 || w >= (int)c.waves.size()) return MW3_ERR_ARG;
    if (w >= (int)c.prodt.size() || !c.prodt[w].on) {
        c.err = "mw3_download_product: the wave has no product projection";
        return MW3_ERR_STATE;
    }
    int rc = build_device(c);
    if (rc) return rc;
    const mw3::ProdDev &d = c.wdev[w].prod;
    if (zs2prod)
        MW3_CUDA_TRY(cudaMemcpyAsync(zs2prod, d.zs2prod, sizeof(double) * 2 * (size_t)d.nrow * c.netot,
                                     cudaMemcpyDeviceToHost, c.stream));
    if (cvjprod)
        MW3_CUDA_TRY(cudaMemcpyAsync(cvjprod, d.cvjprod, sizeof(double) * (size_t)d.nrow, cudaMemcpyDeviceToHost,
                                     c.stream));
    MW3_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return check_device_flags(c, "mw3_download_product");
}

int mw3_upload_product(mw3_ctx *h, int32_t w, const double *zs2prod)
{
    if (!h || !zs2prod) return MW3_ERR_ARG;
    Ctx &c = h->c;
    if (w < 0 || w >= (int)c.waves.size()) return MW3_ERR_ARG;
    if (w >= (int)c.prodt.size() || !c.prodt[w].on || !c.built || !c.started) {
        c.err = "mw3_upload_product: the wave has no product projection, or its state is not uploaded";
        return MW3_ERR_STATE;
    }
    const mw3::ProdDev &d = c.wdev[w].prod;
    MW3_CUDA_TRY(cudaMemcpyAsync(d.zs2prod, zs2prod, sizeof(double) * 2 * (size_t)d.nrow * c.netot,
                                 cudaMemcpyHostToDevice, c.stream));
    MW3_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return MW3_OK;
}

const char *mw3_last_error(const mw3_ctx *h)
{
    if (!h) return "null context";
    return h->c.err.c_str();
}

int mw3_destroy(mw3_ctx *h)
{
    if (!h) return MW3_OK;
    Ctx &c = h->c;
    if (c.stream) cudaStreamSynchronize(c.stream);
    for (cudaEvent_t e : c.prof_ev) cudaEventDestroy(e);
    free_device(c);
    if (c.stream) cudaStreamDestroy(c.stream);
    if (c.h_flag) cudaFreeHost(c.h_flag);
    delete h;
    return MW3_OK;
}

int mw3_set_choices(mw3_ctx *h, const int32_t *choice)
{
    if (!h || !choice) return MW3_ERR_ARG;
    Ctx &c = h->c;
    const int dst = choice[0], xt = choice[1], ang = choice[2], cw = choice[3];
    const bool cw_ok = cw == 0 || (cw >= 8 && cw <= c.ang_cw_fit && (cw & (cw - 1)) == 0);
    if (dst < -1 || dst > (c.fp64 ? 1 : 3) || xt < -1 || xt > 1 || ang < -1 || ang > 1 || !cw_ok) {
        c.err = "mw3_set_choices: choice out of range";
        return MW3_ERR_ARG;
    }
    if (c.started) {
        c.err = "mw3_set_choices: call before mw3_start";
        return MW3_ERR_STATE;
    }
    c.k_dst = dst;
    c.k_xt = xt;
    c.k_ang = ang;
    c.k_cw = cw;
    c.built = false;
    return MW3_OK;
}

int mw3_get_choices(mw3_ctx *h, int32_t *choice)
{
    if (!h || !choice) return MW3_ERR_ARG;
    const Ctx &c = h->c;
    choice[0] = c.k_dst;
    choice[1] = c.k_xt;
    choice[2] = c.k_ang;
    choice[3] = c.k_cw;
    return MW3_OK;
}
}  // extern "C"

namespace {
// what a build with the current choices runs: two builds with one signature run
// the same kernels with the same launch shapes
std::vector<int> path_signature(const Ctx &c)
{
    const bool explicit_ang = c.na > 1 && (c.fp64 || !c.use_tc_ang);
    const bool tc3 = !c.fp64 && !c.use_tc_dst2d && mw3::tc_dst_supported(const_cast<Ctx &>(c));
    return {(int)c.use_tc_dst2d, c.use_tc_dst2d ? (int)c.dst_f16 : -1, (int)tc3, (int)c.use_tc_ang, (int)c.x_t,
            (int)(c.fp64 && c.d_rd_tw != nullptr), explicit_ang ? c.ang_cw : 0};
}

// time n iterations of the propagation from a synthetic state after the warm-up that
// captures both graphs; ms per iteration
int time_candidate(mw3_ctx *h, int n, double *ms)
{
    Ctx &c = h->c;
    mw3::launch_fill_pattern(c, c.d_pk, c.NT);
    int rc = start_device(c);
    if (rc) return rc;
    rc = mw3_run(h, (mw3::kGraphIters - 1) + 2 * mw3::kGraphIters);
    if (rc) return rc;
    cudaEvent_t e0, e1;
    MW3_CUDA_TRY(cudaEventCreate(&e0));
    MW3_CUDA_TRY(cudaEventCreate(&e1));
    cudaEventRecord(e0, c.stream);
    rc = mw3_run(h, n);
    cudaEventRecord(e1, c.stream);
    if (!rc) rc = check_device_flags(c, "mw3_autotune");
    float t = 0.f;
    if (!rc && cudaEventElapsedTime(&t, e0, e1) != cudaSuccess) rc = MW3_ERR_CUDA;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = (double)t / n;
    return rc;
}
}  // namespace

extern "C" int mw3_autotune(mw3_ctx *h, int32_t iterations, int32_t scope, int32_t *choice, double *ms_best)
{
    if (!h || iterations < 1 || scope < 1 || (scope & ~(MW3_TUNE_LAYOUT | MW3_TUNE_FORM))) return MW3_ERR_ARG;
    Ctx &c = h->c;
    if (c.waves.empty()) {
        c.err = "mw3_autotune: no partial wave added";
        return MW3_ERR_STATE;
    }
    if (c.started) {
        c.err = "mw3_autotune: call before mw3_start";
        return MW3_ERR_STATE;
    }
    const int per = 2 * mw3::kGraphIters;
    const int n = (int)(((int64_t)iterations + per - 1) / per) * per;
    const int k0[4] = {c.k_dst, c.k_xt, c.k_ang, c.k_cw};
    std::vector<int> dsts{k0[0]}, angs{k0[2]};
    if (scope & MW3_TUNE_FORM) {
        if (c.fp64) {
            if (c.n2 == 256) dsts = {1, 0};
        } else {
            dsts = {0, 1, 2, 3};
            if (c.na > 1) angs = {1, 0};
        }
    }
    std::vector<std::vector<int>> seen;
    double best = 0.0;
    int bk[4] = {k0[0], k0[1], k0[2], k0[3]};
    bool have = false;
    int rc = MW3_OK;
    for (int d : dsts)
        for (int a : angs) {
            // the layouts this form admits, from a build with the first of them
            c.k_dst = d;
            c.k_ang = a;
            c.k_xt = (scope & MW3_TUNE_LAYOUT) ? 0 : k0[1];
            c.k_cw = (scope & MW3_TUNE_LAYOUT) ? 0 : k0[3];
            c.built = false;
            if ((rc = build_device(c))) goto done;
            std::vector<int> xts{c.k_xt}, cws{c.k_cw};
            if (scope & MW3_TUNE_LAYOUT) {
                if (mw3::xt_eligible(c)) xts = {0, 1};
                if (c.na > 1 && (c.fp64 || !c.use_tc_ang)) {
                    cws.clear();
                    for (int w = c.ang_cw_fit; w >= 8; w /= 2) cws.push_back(w);
                }
            }
            for (int x : xts)
                for (int w : cws) {
                    const bool probe = x == c.k_xt && (w == c.k_cw || (c.k_cw == 0 && w == c.ang_cw_fit));
                    c.k_xt = x;
                    c.k_cw = w;
                    if (!probe) {
                        c.built = false;
                        if ((rc = build_device(c))) goto done;
                    }
                    std::vector<int> sig = path_signature(c);
                    if (std::find(seen.begin(), seen.end(), sig) != seen.end()) continue;
                    seen.push_back(sig);
                    double t = 0.0;
                    if ((rc = time_candidate(h, n, &t))) goto done;
                    if (!have || t < best) {
                        best = t;
                        bk[0] = d; bk[1] = x; bk[2] = a; bk[3] = w;
                        have = true;
                    }
                }
        }
done:
    c.k_dst = rc ? k0[0] : bk[0];
    c.k_xt = rc ? k0[1] : bk[1];
    c.k_ang = rc ? k0[2] : bk[2];
    c.k_cw = rc ? k0[3] : bk[3];
    c.built = false;
    c.started = false;
    if (rc) return rc;
    rc = build_device(c);
    if (rc) return rc;
    if (choice) {
        for (int i = 0; i < 4; i++) choice[i] = bk[i];
    }
    if (ms_best) *ms_best = best;
    return MW3_OK;
}
