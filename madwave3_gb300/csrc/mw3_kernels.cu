// CUDA kernels of the Chebyshev hot path (sm_103a).
//
// One H.psi application (difs, SRC/mod_Hphi_01y2.f:623-943) is five stages over
// every Omega/electronic block of every partial wave at once:
//   1. k_dst_rows   psi rectangle x S2            (DST-I along R, all angles)
//   2. k_dst_cols   S1 (E o (S1 Y))                (DST-I along r twice, k-space scaling between)
//   3. k_dst_rows   Y x S2 with a gather epilogue  (kinetic part at the stored points)
//      k_quirk      stored points with ir1 > nopr1 keep psi (the reference's DST never
//                   reaches them, mod_Hphi_01y2.f:768-831)
//   4. k_ang_j      j^2 part: per r1, dense angle x angle matrix (xj2)
//      k_ang_l      l^2 part incl. Omega+-1 Coriolis coupling: per R (xl2p)
//   5. k_update     V psi, damped three-term recursion, next rectangle, norm partials
// followed by the accumulators (CoefEcheby, totalflux_k, Cvjflux_k).
// T is the transform type: double (plain FP64 path) or float (mixed path); the
// recursion vectors, potential, absorption and accumulators are always FP64.
#include <math.h>
#include <stdio.h>

#include <algorithm>
#include <mutex>

#include "mw3_internal.h"

namespace mw3 {

#define LAUNCH_CHECK(c) do { (c).launches++; } while (0)

// ---------------------------------------------------------------------------
// scatter: compressed psi -> rectangle X[g][a][ir1][ir2]
// ---------------------------------------------------------------------------
constexpr int kPointChunk = 1024;   // stored points per CTA in the point kernels

__device__ __forceinline__ float f64_to_f32_int(double x);
template <typename T> __device__ __forceinline__ T rect_value(double v) { return (T)v; }
// FP32 rectangles take the update kernel's rounding, so a restart reproduces a run
template <> __device__ __forceinline__ float rect_value<float>(double v) { return f64_to_f32_int(v); }

// psi32 (optional): the FP32 copy of psi at the stored points, which the mixed
// update reads for the potential term
template <typename T>
__global__ void k_scatter(DevGrid d, T *__restrict__ X, const double *__restrict__ psi, float *__restrict__ psi32,
                          int seg0, unsigned *__restrict__ xmax)
{
    int seg = seg0 + blockIdx.x;
    int a = seg % d.na;
    int64_t off = d.foff[seg];
    int n = d.npunreal[a];
    int i0 = blockIdx.y * kPointChunk, i1 = min(n, i0 + kPointChunk);
    T *base = X + (size_t)seg * d.n1 * d.n2;
    float m = 0.f;
    for (int ir = i0 + threadIdx.x; ir < i1; ir += blockDim.x) {
        int ir1 = d.indr1[(size_t)a * d.npt + ir] - 1;
        int ir2 = d.indr2[(size_t)a * d.npt + ir] - 1;
        const double v = psi[off + ir];
        const T x = rect_value<T>(v);
        base[d.xt ? (size_t)ir2 * d.n1 + ir1 : (size_t)ir1 * d.n2 + ir2] = x;
        m = fmaxf(m, fabsf((float)x));
        if (psi32) psi32[off + ir] = rect_value<float>(v);
    }
    // the slab's largest |X| for the split-FP16 DST (its scale)
    if (xmax) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMax(xmax + seg, __float_as_uint(m));
    }
}

// ---------------------------------------------------------------------------
// row DST: C[r][:] = A[r][:] x S2 for the rows r = (g, a, ir1) with ir1 < nopr1
// register-tiled GEMM; epilogue either stores C or gathers it into H
// ---------------------------------------------------------------------------
// The DST-I matrices are symmetric and S[n-1-i][k] = (-1)^k S[i][k], so with
// E_i and O_i the sums over even and odd k, y_i = E_i + O_i and
// y_{n-1-i} = E_i - O_i: both transforms compute only the first ceil(n/2)
// outputs, from two accumulators, and mirror them (the first radix-2 level of
// an FFT of the odd extension; the rest stays dense because n + 1 is prime or
// has large factors for the grid lengths in use).  Half the multiply-adds of
// the dense product; the sums run in the same k order within each parity.
template <typename T> struct RowCfg;
template <> struct RowCfg<double> { enum { BM = 64, BN = 64, BK = 16, TM = 4, TN = 4 }; };
template <> struct RowCfg<float> { enum { BM = 128, BN = 64, BK = 16, TM = 8, TN = 4 }; };

// C[r][i] = sum_k A[r][k] S[k][i] over rows r of every slab (DST along R); grid.y
// covers the first ceil(n2/2) output columns, each CTA writing both mirrors
template <typename T, bool GATHER>
__global__ void __launch_bounds__(256) k_dst_rows(DevGrid d, const T *__restrict__ A, const T *__restrict__ S,
                                                  T *__restrict__ C, double *__restrict__ H,
                                                  const int *__restrict__ nopr1, int64_t row0, int64_t nrows)
{
    constexpr int BM = RowCfg<T>::BM, BN = RowCfg<T>::BN, BK = RowCfg<T>::BK;
    constexpr int TM = RowCfg<T>::TM, TN = RowCfg<T>::TN;
    constexpr int TX = BN / TN, TY = BM / TM;
    static_assert(TX * TY == 256, "256 threads");
    static_assert(BK % 2 == 0, "chunks start at even k");
    __shared__ T As[BK][BM + 1];
    __shared__ T Bs[BK][BN];
    const int n1 = d.n1, n2 = d.n2, na = d.na, h = (n2 + 1) / 2;
    int64_t rbase = row0 + (int64_t)blockIdx.x * BM;     // row tiles on x: no 65535 limit
    int cbase = blockIdx.y * BN;
    int tid = threadIdx.x;
    // skip tiles whose rows all lie beyond the DST length of their angle
    __shared__ int any;
    if (tid == 0) any = 0;
    __syncthreads();
    if (tid < BM) {
        int64_t r = rbase + tid;
        if (r < row0 + nrows) {
            int64_t ga = r / n1;
            int ir1 = (int)(r % n1);
            int g = (int)(ga / na), a = (int)(ga % na);
            if (ir1 < nopr1[d.blk_wave[g] * na + a]) any = 1;
        }
    }
    __syncthreads();
    if (!any) return;
    int tx = tid % TX, ty = tid / TX;
    T ae[TM][TN], ao[TM][TN];
#pragma unroll
    for (int m = 0; m < TM; m++)
#pragma unroll
        for (int n = 0; n < TN; n++) ae[m][n] = ao[m][n] = (T)0;
    for (int k0 = 0; k0 < n2; k0 += BK) {
        for (int e = tid; e < BM * BK; e += 256) {
            int i = e / BK, kk = e % BK;
            int64_t r = rbase + i;
            T v = 0;
            if (r < row0 + nrows && k0 + kk < n2) v = A[r * n2 + k0 + kk];
            As[kk][i] = v;
        }
        for (int e = tid; e < BK * BN; e += 256) {
            int kk = e / BN, j = e % BN;
            T v = 0;
            if (k0 + kk < n2 && cbase + j < h) v = S[(size_t)(k0 + kk) * n2 + cbase + j];
            Bs[kk][j] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; kk += 2) {
            T av[TM], bv[TN], aw[TM], bw[TN];
#pragma unroll
            for (int m = 0; m < TM; m++) {
                av[m] = As[kk][ty + m * TY];
                aw[m] = As[kk + 1][ty + m * TY];
            }
#pragma unroll
            for (int n = 0; n < TN; n++) {
                bv[n] = Bs[kk][tx + n * TX];
                bw[n] = Bs[kk + 1][tx + n * TX];
            }
#pragma unroll
            for (int m = 0; m < TM; m++)
#pragma unroll
                for (int n = 0; n < TN; n++) {
                    ae[m][n] += av[m] * bv[n];
                    ao[m][n] += aw[m] * bw[n];
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int m = 0; m < TM; m++) {
        int64_t r = rbase + ty + m * TY;
        if (r >= row0 + nrows) continue;
        int64_t ga = r / n1;
        int ir1 = (int)(r % n1);
        int g = (int)(ga / na), a = (int)(ga % na);
        if (ir1 >= nopr1[d.blk_wave[g] * na + a]) continue;
#pragma unroll
        for (int n = 0; n < TN; n++) {
            int col = cbase + tx + n * TX;
            if (col >= h) continue;
            const int mir = n2 - 1 - col;
            const T y0 = ae[m][n] + ao[m][n], y1 = ae[m][n] - ao[m][n];
            if (GATHER) {
                const int *mp = d.map + ((size_t)a * n1 + ir1) * n2;
                int idx = mp[col];
                if (idx >= 0) H[d.foff[ga] + idx] = (double)y0;
                if (mir != col && (idx = mp[mir]) >= 0) H[d.foff[ga] + idx] = (double)y1;
            } else {
                C[r * n2 + col] = y0;
                if (mir != col) C[r * n2 + mir] = y1;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// column DSTs: for one (block, angle) and a tile of W columns,
// Y[0:nn][cols] <- S1 ( E o (S1 Y[0:nn][cols]) ),  E = min(p2r1+p2r2, radcut)/(4(nn+1)(n2+1))
// each thread sums rows i < ceil(nn/2) by parity of k and writes rows i and nn-1-i
// ---------------------------------------------------------------------------
constexpr int COL_W = 32;
constexpr int COL_KC = 32;
constexpr int COL_RMAX = 16;   // folded rows per thread (n1 <= 256)

template <typename T>
__global__ void __launch_bounds__(256) k_dst_cols(DevGrid d, T *__restrict__ Y, const T *__restrict__ S1all,
                                                  const int64_t *__restrict__ s1off, const int *__restrict__ nopr1,
                                                  const double *__restrict__ p2r1, const double *__restrict__ p2r2,
                                                  double radcut, int seg0)
{
    extern __shared__ unsigned char smraw[];
    T *Yt = reinterpret_cast<T *>(smraw);                 // [n1][COL_W]
    T *Sc = Yt + (size_t)d.n1 * COL_W;                    // [n1][COL_KC]
    int seg = seg0 + blockIdx.x;
    int g = seg / d.na, a = seg % d.na;
    int w = d.blk_wave[g];
    int nn = nopr1[w * d.na + a];
    const int hn = (nn + 1) / 2;
    const T *S1 = S1all + s1off[w * d.na + a];
    int n1 = d.n1, n2 = d.n2;
    int c0 = blockIdx.y * COL_W;
    int tx = threadIdx.x % COL_W, ty = threadIdx.x / COL_W;   // 8 row groups
    T *base = Y + (size_t)seg * n1 * n2;
    for (int e = threadIdx.x; e < nn * COL_W; e += 256) {
        int k = e / COL_W, cc = e % COL_W;
        Yt[k * COL_W + cc] = (c0 + cc < n2) ? base[(size_t)k * n2 + c0 + cc] : (T)0;
    }
    const double *p1 = p2r1 + ((size_t)w * d.na + a) * n1;
    const double *p2 = p2r2 + ((size_t)w * d.na + a) * n2;
    const T divi = (T)(1.0 / (4.0 * (double)(nn + 1) * (double)(n2 + 1)));
    const T rcut = (T)radcut;
    T ae[COL_RMAX], ao[COL_RMAX];
    const int nr = ty < hn ? (hn - 1 - ty) / 8 + 1 : 0;    // rows ty + 8 r < hn of this warp
    for (int pass = 0; pass < 2; pass++) {
#pragma unroll
        for (int r = 0; r < COL_RMAX; r++) ae[r] = ao[r] = (T)0;
        for (int kc = 0; kc < nn; kc += COL_KC) {
            __syncthreads();
            for (int e = threadIdx.x; e < hn * COL_KC; e += 256) {
                int i = e / COL_KC, kk = e % COL_KC;
                Sc[i * COL_KC + kk] = (kc + kk < nn) ? S1[(size_t)i * nn + kc + kk] : (T)0;
            }
            __syncthreads();
            int kmax = min(COL_KC, nn - kc);
            for (int kk = 0; kk < kmax; kk += 2) {
                T y0 = Yt[(kc + kk) * COL_W + tx];
                T y1 = kk + 1 < kmax ? Yt[(kc + kk + 1) * COL_W + tx] : (T)0;
                // a warp's rows end at nr (uniform): leave instead of issuing masked FMAs
#pragma unroll
                for (int r = 0; r < COL_RMAX; r++) {
                    if (r >= nr) break;
                    const T *sr = Sc + (ty + 8 * r) * COL_KC + kk;
                    ae[r] += sr[0] * y0;
                    ao[r] += sr[1] * y1;
                }
            }
        }
        __syncthreads();
        if (pass == 0) {
            int col = c0 + tx;
#pragma unroll
            for (int r = 0; r < COL_RMAX; r++) {
                int i = ty + 8 * r;
                if (i >= hn) continue;
                const int im = nn - 1 - i;
                if (col < n2) {
                    T ek = (T)p1[i] + (T)p2[col];
                    if (ek > rcut) ek = rcut;
                    Yt[i * COL_W + tx] = (ae[r] + ao[r]) * ek * divi;
                    if (im != i) {
                        T em = (T)p1[im] + (T)p2[col];
                        if (em > rcut) em = rcut;
                        Yt[im * COL_W + tx] = (ae[r] - ao[r]) * em * divi;
                    }
                } else {
                    Yt[i * COL_W + tx] = (T)0;
                    Yt[im * COL_W + tx] = (T)0;
                }
            }
        }
    }
    int col = c0 + tx;
    if (col < n2)
#pragma unroll
        for (int r = 0; r < COL_RMAX; r++) {
            int i = ty + 8 * r;
            if (i >= hn) continue;
            const int im = nn - 1 - i;
            base[(size_t)i * n2 + col] = ae[r] + ao[r];
            if (im != i) base[(size_t)im * n2 + col] = ae[r] - ao[r];
        }
}

// ---------------------------------------------------------------------------
// FP64 DST along R for npun2 = 256 as a 257-point transform by Rader's algorithm.
// y_i = sum_k 2 sin(pi i k / 257) x_k (i, k = 1..256) is read off the 257-point DFT W
// of w_k = x_k + i (-1)^k x_k: y_2j = Im W_{257-j} - Im W_j (j <= 128) and
// y_{2j-257} = Re W_j - Re W_{257-j} (j >= 129).  257 is prime with primitive root 3,
// so W_{3^-p} = sum_q w_{3^q} d_{p-q} (indices mod 256, d_m = exp(-2 pi i 3^-m / 257)),
// a 256-point cyclic convolution: FFT, product with d's FFT (a table, / 256), and the
// inverse as conj(FFT(conj(.))); W_{257-j} sits 128 places from W_j (3^128 = -1).  The
// FFTs are radix-4 Stockham passes in shared memory (natural order, no bit reversal).
// About 14 k FP64 operations a row, against 33 k multiply-adds for the folded dense
// product, and only the rows ir1 < nopr1 are transformed (the dense kernel computes
// whole 64-row tiles).  Four rows per CTA batch, one per 64-thread group.
// ---------------------------------------------------------------------------
constexpr int RD_M = 256, RD_ROWS = 4;

__device__ __forceinline__ double2 cmul(double2 a, double2 b)
{
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// forward FFT of a[256] (in place through b), radix-4 Stockham, 64 threads a row
__device__ __forceinline__ void rd_fft256(double2 *a, double2 *b, const double2 *tw, int t)
{
    double2 *in = a, *out = b;
#pragma unroll
    for (int ns = 1; ns < RD_M; ns *= 4) {
        double2 v[4];
#pragma unroll
        for (int r = 0; r < 4; r++) v[r] = in[t + 64 * r];
        if (ns > 1) {
            const int jm = t % ns, st = 64 / ns;
#pragma unroll
            for (int r = 1; r < 4; r++) v[r] = cmul(v[r], tw[jm * r * st]);
        }
        const double2 a0 = make_double2(v[0].x + v[2].x, v[0].y + v[2].y);
        const double2 a1 = make_double2(v[0].x - v[2].x, v[0].y - v[2].y);
        const double2 a2 = make_double2(v[1].x + v[3].x, v[1].y + v[3].y);
        const double2 a3 = make_double2(v[1].x - v[3].x, v[1].y - v[3].y);
        const int d0 = (t / ns) * ns * 4 + t % ns;
        out[d0] = make_double2(a0.x + a2.x, a0.y + a2.y);
        out[d0 + ns] = make_double2(a1.x + a3.y, a1.y - a3.x);        // a1 - i a3
        out[d0 + 2 * ns] = make_double2(a0.x - a2.x, a0.y - a2.y);
        out[d0 + 3 * ns] = make_double2(a1.x - a3.y, a1.y + a3.x);    // a1 + i a3
        __syncthreads();
        double2 *tmp = in;
        in = out;
        out = tmp;
    }
}

struct RaderTab {
    const double2 *tw, *ch;
    const short *col;
    const int *out;
    const int64_t *rowpre;
};

template <bool GATHER>
__global__ void __launch_bounds__(256) k_dst_rows_rader(DevGrid d, const double *__restrict__ A,
                                                        double *__restrict__ C, double *__restrict__ H, RaderTab rt,
                                                        int seg0, int nseg)
{
    __shared__ double2 s_tw[RD_M], s_ch[RD_M];
    __shared__ short s_col[RD_M];
    __shared__ int s_out[RD_M];
    __shared__ double2 s_buf[RD_ROWS][2][RD_M];
    const int tid = threadIdx.x, grp = tid >> 6, t = tid & 63;
    s_tw[tid] = rt.tw[tid];
    s_ch[tid] = rt.ch[tid];
    s_col[tid] = rt.col[tid];
    s_out[tid] = rt.out[tid];
    const int64_t v1 = rt.rowpre[seg0 + nseg];
    const int n1 = d.n1, na = d.na;
    double2 *a = s_buf[grp][0], *b = s_buf[grp][1];
    double *xs = reinterpret_cast<double *>(b);
    for (int64_t vb = rt.rowpre[seg0] + (int64_t)blockIdx.x * RD_ROWS; vb < v1;
         vb += (int64_t)gridDim.x * RD_ROWS) {
        const int64_t v = vb + grp;
        const bool live = v < v1;
        int seg = seg0, ir1 = 0;
        if (live) {
            // the segment holding transformed row v: the last with rowpre[seg] <= v
            int lo = seg0, hi = seg0 + nseg - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (rt.rowpre[mid] <= v) lo = mid;
                else hi = mid - 1;
            }
            seg = lo;
            ir1 = (int)(v - rt.rowpre[seg]);
        }
        const int64_t row = (int64_t)seg * n1 + ir1;
        __syncthreads();                    // the tables, and the previous batch's reads of b
        if (live)
#pragma unroll
            for (int k = 0; k < 4; k++) xs[t + 64 * k] = A[row * RD_M + t + 64 * k];
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int q = t + 64 * k, c = s_col[q];
            const double x = live ? xs[c] : 0.0;
            a[q] = make_double2(x, (c & 1) ? x : -x);   // k = c + 1: (-1)^k x
        }
        __syncthreads();
        rd_fft256(a, b, s_tw, t);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int q = t + 64 * k;
            const double2 z = cmul(a[q], s_ch[q]);
            a[q] = make_double2(z.x, -z.y);
        }
        __syncthreads();
        rd_fft256(a, b, s_tw, t);            // a = FFT(conj(.)): W_{3^-p} = conj(a[p])
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int p = t + 64 * k, q = (p + 128) & (RD_M - 1), o = s_out[p];
            const double y = (o >> 16) ? a[p].x - a[q].x : a[p].y - a[q].y;
            xs[o & 0xffff] = y;
        }
        __syncthreads();
        if (live) {
            if (GATHER) {
                const int ang = seg % na;
                const int *mp = d.map + ((size_t)ang * n1 + ir1) * RD_M;
                const int64_t fo = d.foff[seg];
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const int col = t + 64 * k, idx = mp[col];
                    if (idx >= 0) H[fo + idx] = xs[col];
                }
            } else {
#pragma unroll
                for (int k = 0; k < 4; k++) C[row * RD_M + t + 64 * k] = xs[t + 64 * k];
            }
        }
    }
}

static int rd_grid()
{
    static int g = 0;
    if (!g) {
        int dev = 0, nsm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        g = (nsm > 0 ? nsm : 1) * 5;        // 41.5 KB of shared memory a CTA: five per SM
    }
    return g;
}

static RaderTab rd_tab(const Ctx &c)
{
    RaderTab r;
    r.tw = c.d_rd_tw;
    r.ch = c.d_rd_ch;
    r.col = c.d_rd_col;
    r.out = c.d_rd_out;
    r.rowpre = c.d_rowpre;
    return r;
}

// double -> float, round to nearest even, with integer instructions only (the
// F2F conversion issues on the FP64 pipe); magnitudes below FLT_MIN go to a
// signed zero, above FLT_MAX to infinity
__device__ __forceinline__ float f64_to_f32_int(double x)
{
    unsigned long long b = (unsigned long long)__double_as_longlong(x);
    unsigned int sign = (unsigned int)(b >> 32) & 0x80000000u;
    int e = (int)((b >> 52) & 0x7FF) - 1023 + 127;
    if (e <= 0) return __uint_as_float(sign);
    if (e >= 255) return __uint_as_float(sign | 0x7F800000u);
    unsigned int m = (unsigned int)((b >> 29) & 0x7FFFFFu);
    unsigned int rest = (unsigned int)(b & 0x1FFFFFFFu);
    unsigned int r = ((unsigned int)e << 23) | m;
    if (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) r += 1u;   // carry may round into the exponent
    if (r >= 0x7F800000u) r = 0x7F800000u;
    return __uint_as_float(sign | r);
}

// exact float -> double with integer instructions (the F2F conversion issues
// on the FP64 pipe); subnormal inputs become a signed zero
__device__ __forceinline__ double f32_to_f64_int(float f)
{
    unsigned int u = __float_as_uint(f);
    unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
    unsigned int e = (u >> 23) & 0xFFu, mt = u & 0x7FFFFFu;
    if (e == 0) return __longlong_as_double((long long)sign);
    unsigned long long ex = (e == 255) ? 0x7FFull : (unsigned long long)(e - 127 + 1023);
    return __longlong_as_double((long long)(sign | (ex << 52) | ((unsigned long long)mt << 29)));
}

__device__ __forceinline__ double h_val(double h) { return h; }
__device__ __forceinline__ double h_val(float h) { return f32_to_f64_int(h); }
__device__ __forceinline__ float h_f32(float h) { return h; }
__device__ __forceinline__ float h_f32(double h) { return f64_to_f32_int(h); }
__device__ __forceinline__ double h_load(const double *H, int64_t i) { return H[i]; }
__device__ __forceinline__ double h_load(const float *H, int64_t i) { return f32_to_f64_int(H[i]); }
__device__ __forceinline__ void h_store(double *H, int64_t i, double v) { H[i] = v; }
__device__ __forceinline__ void h_store(float *H, int64_t i, double v) { H[i] = f64_to_f32_int(v); }

// H (FP64) = H32 at every stored point of the segments, for the explicit
// angular kernels that accumulate in FP64
__global__ void k_h32_to_h(DevGrid d, const float *__restrict__ h32, double *__restrict__ H, int seg0)
{
    int seg = seg0 + blockIdx.x;
    int a = seg % d.na;
    int64_t off = d.foff[seg];
    int n = min(d.npunreal[a], (int)(blockIdx.y + 1) * kPointChunk);
    for (int ir = blockIdx.y * kPointChunk + threadIdx.x; ir < n; ir += blockDim.x) H[off + ir] = f32_to_f64_int(h32[off + ir]);
}

// stored points with ir1 beyond the DST length keep psi as their "kinetic" term
template <typename HT>
__global__ void k_quirk(DevGrid d, const double *__restrict__ psi, HT *__restrict__ H,
                        const int *__restrict__ qptr, const int *__restrict__ qlist, int seg0)
{
    int seg = seg0 + blockIdx.x;
    int g = seg / d.na, a = seg % d.na;
    int w = d.blk_wave[g];
    int b = qptr[w * d.na + a], e = qptr[w * d.na + a + 1];
    int64_t off = d.foff[seg];
    for (int q = b + threadIdx.x; q < e; q += blockDim.x) {
        int ir = qlist[q];
        h_store(H, off + ir, psi[off + ir]);
    }
}

// ---------------------------------------------------------------------------
// angular kinetic terms in the grid representation
// ---------------------------------------------------------------------------
// the column chunk of the explicit angular kernels is c.ang_cw (64, or narrower
// when the angle count makes the staged matrices too large for shared memory)

// Target descriptors of one angular CTA: angle, column inside the chunk and
// output index, with eight independent loads in flight per thread.
__device__ __forceinline__ void stage_targets(const DevGrid &d, const int *__restrict__ tl, int nt,
                                              const int *__restrict__ ind, int c0, size_t frow, int *t_a, int *t_c,
                                              long long *t_o)
{
    constexpr int U = 8;
    for (int q0 = threadIdx.x; q0 < nt; q0 += U * blockDim.x) {
        int ent[U], col[U];
        long long off[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            int q = q0 + u * blockDim.x;
            ent[u] = q < nt ? __ldg(tl + q) : 0;
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            int a = ent[u] >> 20, ir = ent[u] & 0xFFFFF;
            col[u] = __ldg(ind + (size_t)a * d.npt + ir) - 1 - c0;
            off[u] = __ldg(d.foff + frow + a) + ir;
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            int q = q0 + u * blockDim.x;
            if (q < nt) {
                t_a[q] = ent[u] >> 20;
                t_c[q] = col[u];
                t_o[q] = off[u];
            }
        }
    }
}

// j^2: H(g, a, r1, r2) += sum_j' X(g, j', r1, r2) xj2(g, r1, a, j')
template <typename T>
__global__ void __launch_bounds__(256) k_ang_j(DevGrid d, const T *__restrict__ X, const T *__restrict__ xj2,
                                               double *__restrict__ H, const int *__restrict__ tptr,
                                               const int *__restrict__ tlist, int ncj, int g0, int ANG_CW)
{
    extern __shared__ unsigned char smraw[];
    int chunk = blockIdx.x, ir1 = blockIdx.y, g = g0 + blockIdx.z;
    int b = tptr[ir1 * ncj + chunk], e = tptr[ir1 * ncj + chunk + 1];
    if (b == e) return;
    int na = d.na, n1 = d.n1, n2 = d.n2;
    T *Xs = reinterpret_cast<T *>(smraw);       // [na][ANG_CW]
    T *xs = Xs + (size_t)na * ANG_CW;           // [na][na+1]
    // target descriptors (angle, column, output index), loaded with all loads in flight
    int *t_a = reinterpret_cast<int *>(xs + (size_t)na * (na + 1));
    int *t_c = t_a + na * ANG_CW;
    long long *t_o = reinterpret_cast<long long *>(t_c + na * ANG_CW);
    stage_targets(d, tlist + b, e - b, d.indr2, chunk * ANG_CW, (size_t)g * na, t_a, t_c, t_o);
    int c0 = chunk * ANG_CW;
    for (int i = threadIdx.x; i < na * ANG_CW; i += blockDim.x) {
        int j = i / ANG_CW, cc = i % ANG_CW;
        Xs[i] = (c0 + cc < n2) ? X[(((size_t)g * na + j) * n1 + ir1) * n2 + c0 + cc] : (T)0;
    }
    const T *xm = xj2 + ((size_t)g * n1 + ir1) * na * na;
    for (int i = threadIdx.x; i < na * na; i += blockDim.x) xs[(i / na) * (na + 1) + (i % na)] = xm[i];
    __syncthreads();
    for (int q = threadIdx.x; q < e - b; q += blockDim.x) {
        int col = t_c[q];
        T acc = (T)0;
        const T *row = xs + (size_t)t_a[q] * (na + 1);
        for (int j = 0; j < na; j++) acc += Xs[j * ANG_CW + col] * row[j];
        H[t_o[q]] += (double)acc;
    }
}

// electronic Coriolis coupling (mod_Hphi_eCoriolis_01y2.f:901-911): for each target
// block t of the list, H(t, a, r1, r2) += sum_s sum_j' X(s, j', r1, r2) xj2e(m, r1, a, j')
// over its source blocks s (equal Omega, Lambda one apart) with m the pair's matrix;
// one CTA per (R chunk, r1, target) sums every source before its single update of H
template <typename T, typename HT>
__global__ void __launch_bounds__(256) k_ang_je(DevGrid d, const T *__restrict__ X, const T *__restrict__ xj2e,
                                                HT *__restrict__ H, const int *__restrict__ tptr,
                                                const int *__restrict__ tlist, int ncj, const int *__restrict__ tgt,
                                                const int *__restrict__ esrc, const int *__restrict__ emat,
                                                int nslot, int ANG_CW)
{
    extern __shared__ unsigned char smraw[];
    int chunk = blockIdx.x, ir1 = blockIdx.y, z = blockIdx.z;
    int b = tptr[ir1 * ncj + chunk], e = tptr[ir1 * ncj + chunk + 1];
    if (b == e) return;
    int na = d.na, n1 = d.n1, n2 = d.n2, g = tgt[z];
    T *acc = reinterpret_cast<T *>(smraw);                     // [e-b]
    T *Xs = reinterpret_cast<T *>(acc + (na * ANG_CW));         // [na][ANG_CW]
    T *xs = Xs + (size_t)na * ANG_CW;                           // [na][na+1]
    int *t_a = reinterpret_cast<int *>(xs + (size_t)na * (na + 1));
    int *t_c = t_a + na * ANG_CW;
    long long *t_o = reinterpret_cast<long long *>(t_c + na * ANG_CW);
    int c0 = chunk * ANG_CW;
    int nt = e - b;
    for (int q = threadIdx.x; q < nt; q += blockDim.x) acc[q] = (T)0;
    stage_targets(d, tlist + b, nt, d.indr2, c0, (size_t)g * na, t_a, t_c, t_o);
    for (int slot = 0; slot < nslot; slot++) {
        int s = esrc[z * nslot + slot], m = emat[z * nslot + slot];
        if (s < 0) continue;
        __syncthreads();
        for (int i = threadIdx.x; i < na * ANG_CW; i += blockDim.x) {
            int j = i / ANG_CW, cc = i % ANG_CW;
            Xs[i] = (c0 + cc < n2) ? X[(((size_t)s * na + j) * n1 + ir1) * n2 + c0 + cc] : (T)0;
        }
        const T *xm = xj2e + ((size_t)m * n1 + ir1) * na * na;
        for (int i = threadIdx.x; i < na * na; i += blockDim.x) xs[(i / na) * (na + 1) + (i % na)] = xm[i];
        __syncthreads();
        for (int q = threadIdx.x; q < nt; q += blockDim.x) {
            int col = t_c[q];
            T s_ = (T)0;
            const T *row = xs + (size_t)t_a[q] * (na + 1);
            for (int j = 0; j < na; j++) s_ += Xs[j * ANG_CW + col] * row[j];
            acc[q] += s_;
        }
    }
    __syncthreads();
    for (int q = threadIdx.x; q < nt; q += blockDim.x) H[t_o[q]] += (HT)acc[q];
}

// l^2 with Omega coupling: H(t, a, r1, r2) += sum_(s,q) sum_j' X(s, j', r1, r2) xl2p(s, q, r2, a, j')
template <typename T>
__global__ void __launch_bounds__(256) k_ang_l(DevGrid d, const T *__restrict__ X, const T *__restrict__ xl2p,
                                               double *__restrict__ H, const int *__restrict__ tptr,
                                               const int *__restrict__ tlist, const int *__restrict__ cpl, int ncl,
                                               int g0, int ANG_CW)
{
    extern __shared__ unsigned char smraw[];
    int chunk = blockIdx.x, ir2 = blockIdx.y, t = g0 + blockIdx.z;
    int b = tptr[ir2 * ncl + chunk], e = tptr[ir2 * ncl + chunk + 1];
    if (b == e) return;
    int na = d.na, n1 = d.n1, n2 = d.n2;
    T *acc = reinterpret_cast<T *>(smraw);                     // [e-b]
    T *Xs = reinterpret_cast<T *>(acc + (na * ANG_CW));         // [na][ANG_CW]
    T *xs = Xs + (size_t)na * ANG_CW;                           // [na][na+1]
    int *t_a = reinterpret_cast<int *>(xs + (size_t)na * (na + 1));
    int *t_c = t_a + na * ANG_CW;
    long long *t_o = reinterpret_cast<long long *>(t_c + na * ANG_CW);
    int c0 = chunk * ANG_CW;
    int nt = e - b;
    for (int q = threadIdx.x; q < nt; q += blockDim.x) acc[q] = (T)0;
    stage_targets(d, tlist + b, nt, d.indr1, c0, (size_t)t * na, t_a, t_c, t_o);
    for (int slot = 0; slot < 3; slot++) {
        int s = cpl[(t * 3 + slot) * 2], qq = cpl[(t * 3 + slot) * 2 + 1];
        if (s < 0) continue;
        __syncthreads();
        for (int i = threadIdx.x; i < na * ANG_CW; i += blockDim.x) {
            int j = i / ANG_CW, cc = i % ANG_CW;
            Xs[i] = (c0 + cc < n1) ? X[(((size_t)s * na + j) * n1 + c0 + cc) * n2 + ir2] : (T)0;
        }
        const T *xm = xl2p + (((size_t)s * 3 + (qq + 1)) * n2 + ir2) * na * na;
        for (int i = threadIdx.x; i < na * na; i += blockDim.x) xs[(i / na) * (na + 1) + (i % na)] = xm[i];
        __syncthreads();
        for (int q = threadIdx.x; q < nt; q += blockDim.x) {
            int col = t_c[q];
            T s_ = (T)0;
            const T *row = xs + (size_t)t_a[q] * (na + 1);
            for (int j = 0; j < na; j++) s_ += Xs[j * ANG_CW + col] * row[j];
            acc[q] += s_;
        }
    }
    __syncthreads();
    for (int q = threadIdx.x; q < nt; q += blockDim.x) H[t_o[q]] += (double)acc[q];
}

// ---------------------------------------------------------------------------
// potential, damped Chebyshev recursion (main_madwave3.f:332-339, first step
// :245-248), next rectangle, norm partials and funE (mod_PsiE_01y2.f:108-120)
// ---------------------------------------------------------------------------
struct UpdArgs {
    const void *H;                 // double, or float when the mixed path keeps H psi in FP32
    const double *pk, *pkm1;
    double *out;
    const int *vsrc;               // [G][ne]
    const double *absfr1, *absfr2; // [W][n1], [W][n2]
    const float *absfr1f, *absfr2f; // FP32 copies (mixed path)
    const int *abs_start;           // [W][2]: first r1 / R index inside an absorber (mixed path)
    double emindlt, delta2;
    double rdelta, r2delta;        // 1/delta2 and 2/delta2 (mixed path)
    const float *vr32;             // mixed path: V 2/delta2 - [same state] emindlt 2/delta2, layout of vvv
    const float *pk32;             // mixed path: FP32 copy of psi_k
    float *out32;                  // mixed path: FP32 copy of psi_k+1
    float r2df;                    // 2/delta2 in FP32
    const UpdChunk *desc;          // non-empty (segment, chunk) pairs, tables resolved
    int nchunk;                    // chunks per segment (norm-partial stride)
    int first;
    double *normpart;              // [G*na]
    int nofe;                      // max over waves; 0 = funE off
    const double *zcke;            // [W][nofe][2]
    double *const *zfe;            // per wave [nofe][ntot_w][2] (null when the wave has none)
    const int64_t *wflat0;         // [W+1]
    unsigned *xmax;                // mixed path: bits of each slab's largest |X| (split-FP16 DST scale)
};

// funE: zfe[e][i] += zcke[w][e] psi_k+1(i) for the selected energies
__device__ __forceinline__ void upd_fe(const UpdArgs &u, double *zf, int w, int64_t wst, int64_t wlen, int64_t i,
                                       double nv)
{
    for (int e = 0; e < u.nofe; e++) {
        const double *ck = u.zcke + ((size_t)w * u.nofe + e) * 2;
        double *zz = zf + ((size_t)e * wlen + (i - wst)) * 2;
        zz[0] += ck[0] * nv;
        zz[1] += ck[1] * nv;
    }
}

// one CTA per non-empty (segment, chunk) pair of the list (angles hold different
// numbers of stored points, so a full segment x chunk grid is a third empty); the
// pair's descriptor carries the table entries, so every thread starts its point
// loads after one independent 48-byte load
template <typename T, typename HT>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 3) k_update(DevGrid d, UpdArgs u, T *__restrict__ X)
{
    const UpdChunk cd = u.desc[blockIdx.x];
    const int seg = cd.seg, chunk = cd.chunk_ns & 255, nsrc = cd.chunk_ns >> 8;
    const int a = cd.wa & 255, w = cd.wa >> 8;
    const int64_t off = cd.off;
    const int n = cd.n;
    const int n1 = d.n1, n2 = d.n2, ne = d.ne;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // same-Omega sources of V psi for this segment: offsets of the potential row and
    // of the psi_k row; the first from the descriptor, a second or later one (several
    // electronic states) from the tables
    __shared__ long long s_voff[8], s_poff[8];
    __shared__ double s_wsum[8];
    if (nsrc > 1) {
        if (threadIdx.x == 0) {
            const int g = seg / d.na, et = d.blk_elec[g];
            int ns = 0;
            for (int q = 0; q < ne; q++) {
                int sb = u.vsrc[g * ne + q];
                if (sb < 0) continue;
                int es = d.blk_elec[sb];
                s_voff[ns] = ((((long long)(et - 1) * ne + (es - 1)) * d.na) + a) * d.npt;
                s_poff[ns] = d.foff[(size_t)sb * d.na + a];
                ns++;
            }
        }
        __syncthreads();
    }
    const HT *__restrict__ Hp = reinterpret_cast<const HT *>(u.H) + off;
    const double *__restrict__ pkp = u.pk + off;
    const double *__restrict__ pm1 = u.pkm1 + off;
    double *__restrict__ outp = u.out + off;
    const int *__restrict__ i1p = d.indr1 + (size_t)a * d.npt;
    const int *__restrict__ i2p = d.indr2 + (size_t)a * d.npt;
    const double *__restrict__ ab1 = u.absfr1 + (size_t)w * n1;
    const double *__restrict__ ab2 = u.absfr2 + (size_t)w * n2;
    T *__restrict__ rect = X + (size_t)seg * n1 * n2;
    const double emin = u.emindlt;
    double nrm = 0.0;
    double *zf = (u.nofe > 0 && !u.first) ? u.zfe[w] : nullptr;
    int64_t wst = u.wflat0[w], wlen = u.wflat0[w + 1] - u.wflat0[w];
    constexpr int U = kPointChunk / 256;        // points per thread, loads issued together
    const int ir0 = chunk * kPointChunk + threadIdx.x;
    float nrmf = 0.f, xmf = 0.f;
    if constexpr (sizeof(T) == 8) {
        int r1[U], r2[U];
        double hv[U], pk[U], p1[U];
#pragma unroll
        for (int k = 0; k < U; k++) {
            int ir = ir0 + k * 256;
            bool on = ir < n;
            r1[k] = on ? i1p[ir] - 1 : 0;
            r2[k] = on ? i2p[ir] - 1 : 0;
            hv[k] = on ? h_load(Hp, ir) : 0.0;
            pk[k] = on ? pkp[ir] : 0.0;
            p1[k] = on && !u.first ? pm1[ir] : 0.0;
        }
        for (int q = 0; q < nsrc; q++) {
            const double *vr = d.vvv + (q == 0 ? cd.voff : s_voff[q]), *pr = u.pk + (q == 0 ? cd.poff : s_poff[q]);
#pragma unroll
            for (int k = 0; k < U; k++) {
                int ir = ir0 + k * 256;
                if (ir < n) hv[k] += pr[ir] * vr[ir];
            }
        }
#pragma unroll
        for (int k = 0; k < U; k++) {
            int ir = ir0 + k * 256;
            if (ir >= n) continue;
            // FP64 path: the reference's operations in its order
            double nv;
            if (u.first) {
                nv = (hv[k] - emin * pk[k]) / u.delta2;
            } else {
                double fab = ab1[r1[k]] * ab2[r2[k]];
                double rhn = (hv[k] - emin * pk[k]) / u.delta2;
                nv = (2.0 * rhn - fab * p1[k]) * fab;
            }
            rect[d.xt ? (size_t)r2[k] * n1 + r1[k] : (size_t)r1[k] * n2 + r2[k]] = (T)nv;
            nrm += nv * nv;
            outp[ir] = nv;
            if (zf) upd_fe(u, zf, w, wst, wlen, off + ir, nv);
        }
    } else {
        // mixed path: the FP64 pipe of GB300 is narrow (the FP64 recursion kept it two
        // thirds busy), so everything that is H psi stays in FP32 and only the
        // recursion itself is FP64:
        //   t = H 2/delta2 + sum_s vr_s psi32_s          (FP32: H psi and V psi)
        //   psi_k+1 = (t - psi_k-1) + d                  (one FP64 add, and a second inside the absorbers)
        //   d = (f - 1) t + (1 - f^2) psi_k-1             (FP32; f the absorption, 0 outside the absorbers)
        // so that psi_k+1 = f t - f^2 psi_k-1 = (t - f psi_k-1) f to FP32 accuracy in d;
        // a warp then runs one FP64 add, or two, instead of both branches of a
        // damped/undamped split.  The FP32 copies of psi_k are read and of psi_k+1
        // written beside the FP64 vectors, the conversions done with integer
        // instructions, the norm in FP32
        const float *vr0 = nsrc > 0 ? u.vr32 + cd.voff : nullptr, *pr0 = nsrc > 0 ? u.pk32 + cd.poff : nullptr;
        const int as1 = u.abs_start[2 * w], as2 = u.abs_start[2 * w + 1];
        float *__restrict__ o32 = u.out32 + off;
        int r1[U], r2[U];
        float hr[U], v0[U], q0[U];
        double p1[U];
#pragma unroll
        for (int k = 0; k < U; k++) {
            int ir = ir0 + k * 256;
            bool on = ir < n;
            r1[k] = on ? i1p[ir] - 1 : 0;
            r2[k] = on ? i2p[ir] - 1 : 0;
            hr[k] = on ? h_f32(Hp[ir]) : 0.f;
            v0[k] = on && vr0 ? vr0[ir] : 0.f;
            q0[k] = on && pr0 ? pr0[ir] : 0.f;
            p1[k] = on && !u.first ? pm1[ir] : 0.0;
        }
#pragma unroll
        for (int k = 0; k < U; k++) {
            int ir = ir0 + k * 256;
            if (ir >= n) continue;
            float acc = v0[k] * q0[k];
            for (int q = 1; q < nsrc; q++) acc = fmaf(u.vr32[s_voff[q] + ir], u.pk32[s_poff[q] + ir], acc);
            const float t32 = fmaf(hr[k], u.r2df, acc);
            double nv;
            if (u.first) {
                nv = f32_to_f64_int(0.5f * t32);
            } else {
                nv = f32_to_f64_int(t32) - p1[k];
                // the absorption factors only where a point can be inside an absorber
                if (r1[k] >= as1 || r2[k] >= as2) {
                    const float a1 = u.absfr1f[(size_t)w * n1 + r1[k]], a2 = u.absfr2f[(size_t)w * n2 + r2[k]];
                    if (!(__float_as_uint(a1) == 0x3F800000u && __float_as_uint(a2) == 0x3F800000u)) {
                        const float f = a1 * a2, p1f = f64_to_f32_int(p1[k]);
                        nv += f32_to_f64_int(fmaf(f - 1.f, t32, (1.f - f * f) * p1f));
                    }
                }
            }
            float nf = f64_to_f32_int(nv);
            // with the transposed rectangle a warp's points (an r1 run) store contiguously
            rect[d.xt ? (size_t)r2[k] * n1 + r1[k] : (size_t)r1[k] * n2 + r2[k]] = (T)nf;
            o32[ir] = nf;
            nrmf = fmaf(nf, nf, nrmf);
            xmf = fmaxf(xmf, fabsf(nf));
            outp[ir] = nv;
            if (zf) upd_fe(u, zf, w, wst, wlen, off + ir, nv);
        }
    }
    if (sizeof(T) == 4 && u.xmax) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) xmf = fmaxf(xmf, __shfl_xor_sync(0xffffffffu, xmf, o));
        if (lane == 0 && xmf > 0.f) atomicMax(u.xmax + seg, __float_as_uint(xmf));
    }
    // norm partial: fixed shuffle tree per warp, then the warps in order (deterministic);
    // the mixed path reduces its FP32 sums in FP32 up to the warp level
    if (sizeof(T) == 4) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) nrmf += __shfl_down_sync(0xffffffffu, nrmf, o);
        nrm = f32_to_f64_int(nrmf);
    } else {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) nrm += __shfl_down_sync(0xffffffffu, nrm, o);
    }
    if (lane == 0) s_wsum[warp] = nrm;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) t += s_wsum[i];
        u.normpart[(size_t)seg * u.nchunk + chunk] = t;
    }
}

// V psi alone, for mw3_hphi: H(t) += sum_s V(e_s, e_t) psi(s) over same-Omega blocks
// (difs V part, mod_Hphi_01y2.f:838-853)
template <typename HT>
// Hin and H may be the same array (each element is read, then written, by one thread)
__global__ void k_addv(DevGrid d, const double *__restrict__ psi, const HT *Hin, double *H,
                       const int *__restrict__ vsrc, int seg0)
{
    int seg = seg0 + blockIdx.x;
    int g = seg / d.na, a = seg % d.na;
    int et = d.blk_elec[g];
    int64_t off = d.foff[seg];
    int n = min(d.npunreal[a], (int)(blockIdx.y + 1) * kPointChunk);
    for (int ir = blockIdx.y * kPointChunk + threadIdx.x; ir < n; ir += blockDim.x) {
        double hv = h_load(Hin, off + ir);
        for (int q = 0; q < d.ne; q++) {
            int s = vsrc[g * d.ne + q];
            if (s < 0) continue;
            int es = d.blk_elec[s];
            double v = d.vvv[((((size_t)(et - 1) * d.ne + (es - 1)) * d.na) + a) * d.npt + ir];
            hv += psi[d.foff[(size_t)s * d.na + a] + ir] * v;
        }
        H[off + ir] = hv;
    }
}

// check (main_madwave3.f:431-442): sum the norm partials of each wave
// base (optional): graph replays read the slot as base[1] + slot
__global__ void k_norms(const double *__restrict__ part, const int *__restrict__ wseg0, const int *__restrict__ wseg1,
                        int nchunk, double *const *norms_out, const int64_t *__restrict__ cap, int64_t slot,
                        const int64_t *__restrict__ base)
{
    if (base) slot += base[1];
    int w = blockIdx.x;
    __shared__ double red[256];
    double s = 0.0;
    for (int64_t i = (int64_t)wseg0[w] * nchunk + threadIdx.x; i < (int64_t)wseg1[w] * nchunk; i += blockDim.x)
        s += part[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0 && slot >= 0 && slot < cap[w]) norms_out[w][slot] = red[0];
}

// ---------------------------------------------------------------------------
// accumulators
// ---------------------------------------------------------------------------
// CoefEcheby (main_madwave3.f:462-490): C_k(E) = d hbar/Delta e^{-ik acos Es}/sqrt(1-Es^2)
// base (optional): graph replays read the iteration as base[0] + k
__global__ void k_coefecheby(const double *__restrict__ etot, int netot, double emindlt, double delta2,
                             double hbr, int64_t k, double *__restrict__ zck, float *__restrict__ cring,
                             int cring_zero, float *__restrict__ cvring, const int64_t *__restrict__ base)
{
    if (base) k += base[0];
    int ie = blockIdx.x * blockDim.x + threadIdx.x;
    if (ie >= netot) return;
    double dd = (k == 0) ? 1.0 : 2.0;
    double zf = dd * hbr / delta2;
    double Es = (etot[ie] - emindlt) / delta2;
    double expo = -(double)k * acos(Es);
    double deno = sqrt(1.0 - Es * Es);
    double s, c;
    sincos(expo, &s, &c);
    zck[2 * ie] = zf * c / deno;
    zck[2 * ie + 1] = zf * s / deno;
    if (cring) {                    // mixed path: this iteration's slot of the flux ring (0: no flux sample)
        float *q = cring + (size_t)(k % kFluxSlots) * netot * 2;
        q[2 * ie] = cring_zero ? 0.f : (float)(zf * c / deno);
        q[2 * ie + 1] = cring_zero ? 0.f : (float)(zf * s / deno);
    }
    if (cvring) {                   // mixed path: this iteration's slot of the Cvj ring
        cvring[2 * ie] = (float)(zf * c / deno);
        cvring[2 * ie + 1] = (float)(zf * s / deno);
    }
}

// totalflux_k (mod_flux_01y2.f:585-660), first half: psi and d psi/d r1 at every
// flux point of every wave; one warp per flux point, lanes stride over the
// stored points of its (block, angle, R) line, butterfly reduction
__global__ void __launch_bounds__(256) k_flux_deriv(const double *__restrict__ psi, const int64_t *__restrict__ fidx,
                                                    const int *__restrict__ dptr, const int64_t *__restrict__ didx,
                                                    const int *__restrict__ dir1, const double *__restrict__ zar,
                                                    int NF, double *__restrict__ fpsi, float *__restrict__ fring,
                                                    const float *__restrict__ psi32, const float *__restrict__ zar32,
                                                    const int *__restrict__ rptr, const int4 *__restrict__ runs,
                                                    int64_t it, const int64_t *__restrict__ base)
{
    int f = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (f >= NF) return;
    if (fring) {
        if (base) it += base[0];
        fring += (size_t)(it % kFluxSlots) * NF * 3;   // this iteration's slot
        // mixed path: FP32 products and sums (the ring holds FP32 anyway) from the FP32
        // copy of psi; with runs (consecutive points and r1) no per-term index is read.
        // Either way lane l takes the line's terms l, l + 32, ... in order.
        float sr = 0.f, si = 0.f;
        const int q0 = dptr[f], q1 = dptr[f + 1];
        if (runs) {
            int qs = 0;                                     // the run's first term within the line
            for (int r = rptr[f]; r < rptr[f + 1]; r++) {
                const int4 rn = runs[r];
                const int64_t st = (int64_t)(((unsigned long long)(unsigned)rn.y << 32) | (unsigned)rn.x);
                for (int q = qs + ((lane - qs) & 31); q < qs + rn.w; q += 32) {
                    const float v = psi32[st + (q - qs)];
                    const int ir1 = rn.z + (q - qs);
                    sr = fmaf(zar32[2 * ir1], v, sr);
                    si = fmaf(zar32[2 * ir1 + 1], v, si);
                }
                qs += rn.w;
            }
        } else {
            for (int q = q0 + lane; q < q1; q += 32) {
                const float v = psi32[didx[q]];
                const int ir1 = dir1[q];
                sr = fmaf(zar32[2 * ir1], v, sr);
                si = fmaf(zar32[2 * ir1 + 1], v, si);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            sr += __shfl_xor_sync(0xffffffffu, sr, o);
            si += __shfl_xor_sync(0xffffffffu, si, o);
        }
        if (lane == 0) {
            fring[3 * (size_t)f] = psi32[fidx[f]];
            fring[3 * (size_t)f + 1] = sr;
            fring[3 * (size_t)f + 2] = si;
        }
        return;
    }
    double sr = 0.0, si = 0.0;
    for (int q = dptr[f] + lane; q < dptr[f + 1]; q += 32) {
        double p = psi[didx[q]];
        int ir1 = dir1[q];
        sr += zar[2 * ir1] * p;
        si += zar[2 * ir1 + 1] * p;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sr += __shfl_xor_sync(0xffffffffu, sr, o);
        si += __shfl_xor_sync(0xffffffffu, si, o);
    }
    if (lane == 0) {
        double p0 = psi[fidx[f]];
        {
            fpsi[4 * (size_t)f] = p0;
            fpsi[4 * (size_t)f + 1] = sr;
            fpsi[4 * (size_t)f + 2] = si;
        }
    }
}

// second half: zCR(E,f) += C_k(E) psi(f), zCdR(E,f) += C_k(E) dpsi(f) for E > V(f)
constexpr int kFluxPerBlock = 8;
__global__ void __launch_bounds__(128) k_flux_acc(const double *__restrict__ fpsi, const double *__restrict__ poti,
                                                  const double *__restrict__ etot, const double *__restrict__ zck,
                                                  int netot, int NF, double *__restrict__ zcr, double *__restrict__ zcdr)
{
    int ie = blockIdx.y * blockDim.x + threadIdx.x;      // flux groups on x: no 65535 limit
    if (ie >= netot) return;
    double e = etot[ie], cr = zck[2 * ie], ci = zck[2 * ie + 1];
    int f0 = blockIdx.x * kFluxPerBlock, f1 = min(NF, f0 + kFluxPerBlock);
    for (int f = f0; f < f1; f++) {
        if (!(e > poti[f])) continue;
        double pf = fpsi[4 * (size_t)f], dr = fpsi[4 * (size_t)f + 1], di = fpsi[4 * (size_t)f + 2];
        size_t o = ((size_t)f * netot + ie) * 2;
        double2 a = *reinterpret_cast<double2 *>(zcr + o);
        double2 b = *reinterpret_cast<double2 *>(zcdr + o);
        a.x += cr * pf;
        a.y += ci * pf;
        b.x += cr * dr - ci * di;
        b.y += cr * di + ci * dr;
        *reinterpret_cast<double2 *>(zcr + o) = a;
        *reinterpret_cast<double2 *>(zcdr + o) = b;
    }
}

// Mixed path: the flux accumulation zCR(E,f) += sum_k C_k(E) psi_k(f) and
// zCdR(E,f) += sum_k C_k(E) dpsi_k(f) for E > V(f), through a ring of the last
// S = kFluxSlots iterations (slot = iteration mod S).  The flux points are cut into
// P = S / q slices of `chunk` points; slice p is flushed over all slots (its last S
// iterations) at the iterations k with k mod S = p q + q - 1, so every (point,
// iteration) is added exactly once and the cost is spread evenly (one slice every
// q iterations).  Products and the sum over the slots in FP32 (a 64 x 64 (E, f)
// tile per CTA, 4 x 4 per thread), added once to the FP64 accumulators.
// final != 0: every slice's iterations since its last flush (slice p: the slots
// with (now - s) mod S < (now - p q - q + 1) mod S), before the accumulators are
// read; the host then clears the C ring, so no iteration is added twice.
constexpr int kFlushE = 64, kFlushF = 64, kFlushS = 32;
__global__ void __launch_bounds__(256) k_flux_flush(const float *__restrict__ fring, const float *__restrict__ cring,
                                                    const double *__restrict__ poti,
                                                    const double *__restrict__ etot, int netot, int NF, int chunk,
                                                    int q, int64_t now, const int64_t *__restrict__ base, int final_,
                                                    double *__restrict__ zcr, double *__restrict__ zcdr)
{
    __shared__ float sc[kFlushS][kFlushE][2];
    __shared__ float sp[kFlushS][kFlushF][3];
    if (base) now += base[0];
    const int nowm = (int)(now % kFluxSlots);
    int f0, f1;
    if (final_) {
        f0 = blockIdx.x * kFlushF;
        f1 = min(NF, f0 + kFlushF);
    } else {
        const int p = nowm / q;
        f0 = p * chunk + blockIdx.x * kFlushF;
        f1 = min(min(NF, (p + 1) * chunk), f0 + kFlushF);
    }
    if (f0 >= f1) return;
    const int e0 = blockIdx.y * kFlushE;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;   // E = e0 + tx + 16 i, f = f0 + ty + 16 j
    float ar[4][4], ai[4][4], br[4][4], bi[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) ar[i][j] = ai[i][j] = br[i][j] = bi[i][j] = 0.f;
    for (int s0 = 0; s0 < kFluxSlots; s0 += kFlushS) {
        // the tile's 4-byte pieces by cp.async (zero-filled outside the slice or the
        // energies), all in flight at once
        constexpr int kNC = kFlushS * kFlushE * 2 / 256, kNP = kFlushS * kFlushF * 3 / 256;
        const uint32_t sc_s = (uint32_t)__cvta_generic_to_shared(&sc[0][0][0]);
        const uint32_t sp_s = (uint32_t)__cvta_generic_to_shared(&sp[0][0][0]);
        __syncthreads();            // the previous chunk's reads of sc / sp are done
#pragma unroll 4
        for (int k = 0; k < kNC; k++) {
            const int i = threadIdx.x + 256 * k, s = i / (kFlushE * 2), r = i % (kFlushE * 2);
            const int e = e0 + r / 2;
            const bool ok = e < netot;
            const float *src = ok ? cring + ((size_t)(s0 + s) * netot + e) * 2 + (r & 1) : cring;
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(sc_s + 4 * i), "l"(src),
                         "r"(ok ? 4 : 0)
                         : "memory");
        }
#pragma unroll 4
        for (int k = 0; k < kNP; k++) {
            const int i = threadIdx.x + 256 * k, s = i / (kFlushF * 3), r = i % (kFlushF * 3);
            const int f = f0 + r / 3;
            const bool ok = f < f1;
            const float *src = ok ? fring + ((size_t)(s0 + s) * NF + f) * 3 + r % 3 : fring;
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(sp_s + 4 * i), "l"(src),
                         "r"(ok ? 4 : 0)
                         : "memory");
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
        asm volatile("cp.async.wait_all;" ::: "memory");
        if (final_) {               // this thread's own pieces outside its slice's window
            for (int k = 0; k < kNP; k++) {
                const int i = threadIdx.x + 256 * k, s = i / (kFlushF * 3), r = i % (kFlushF * 3);
                const int f = f0 + r / 3;
                if (f >= f1) continue;
                const int p = f / chunk;
                const int np = ((nowm - p * q - q + 1) % kFluxSlots + kFluxSlots) % kFluxSlots;
                if ((nowm - (s0 + s) + kFluxSlots) % kFluxSlots >= np) sp[s][r / 3][r % 3] = 0.f;
            }
        }
        __syncthreads();
        for (int s = 0; s < kFlushS; s++) {
            float cr[4], ci[4], p[4], dr[4], di[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                cr[i] = sc[s][tx + 16 * i][0];
                ci[i] = sc[s][tx + 16 * i][1];
            }
#pragma unroll
            for (int j = 0; j < 4; j++) {
                p[j] = sp[s][ty + 16 * j][0];
                dr[j] = sp[s][ty + 16 * j][1];
                di[j] = sp[s][ty + 16 * j][2];
            }
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    ar[i][j] = fmaf(cr[i], p[j], ar[i][j]);
                    ai[i][j] = fmaf(ci[i], p[j], ai[i][j]);
                    br[i][j] = fmaf(cr[i], dr[j], fmaf(-ci[i], di[j], br[i][j]));
                    bi[i][j] = fmaf(cr[i], di[j], fmaf(ci[i], dr[j], bi[i][j]));
                }
        }
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
        int f = f0 + ty + 16 * j;
        if (f >= f1) continue;
        double v = poti[f];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            int e = e0 + tx + 16 * i;
            if (e >= netot || !(etot[e] > v)) continue;
            size_t o = ((size_t)f * netot + e) * 2;
            double2 a = *reinterpret_cast<double2 *>(zcr + o);
            double2 b = *reinterpret_cast<double2 *>(zcdr + o);
            a.x += (double)ar[i][j];
            a.y += (double)ai[i][j];
            b.x += (double)br[i][j];
            b.y += (double)bi[i][j];
            *reinterpret_cast<double2 *>(zcr + o) = a;
            *reinterpret_cast<double2 *>(zcdr + o) = b;
        }
    }
}

// Cvjflux_k (mod_flux_01y2.f:663-775) in three parallel passes over every block
// 1. xj(g, r1, j) = sum_gamma psi(g, gamma, r1, R(ir2abs)) / sqrt(ah2) Djmmp(gamma, j)
struct CvjArgs {
    const double *psi;
    const int *r2abs;             // [W][na][n1]
    const double *djall;
    const int64_t *djoff;         // [W]
    const int *wnangu2;           // [W]
    const int *blk_j00, *blk_inc, *blk_isref;
    const double *fd;             // [nelec][nj][nv][n1]
    const int *nobc;              // [nelec][nj]
    double *xj, *cvj, *zs2;
    const double *zck;
    // mixed path
    const float *pk32, *dj32, *fd32;
    float *xj32, *ring;           // ring: this iteration's slot [G nj nv]
    float rsah2f;
    int jini, jmax, nvini, nvmax, nj, nv, netot, jref, nvref, gate;
    double sah2;
};

__device__ inline bool cvj_on(const CvjArgs &c, int g, int j) { return j >= c.blk_j00[g] && ((j - c.blk_j00[g]) % c.blk_inc[g]) == 0; }

constexpr int kCvjR1 = 8;   // r1 points per CTA of the Cvj projection

__global__ void __launch_bounds__(256) k_cvj_proj(DevGrid d, CvjArgs c)
{
    // one CTA per block: gather psi on the line R = R(ir2abs) for every angle and
    // the block's Djmmp columns into shared memory, then contract over angles
    extern __shared__ double cvsm[];
    int g = blockIdx.x;
    int n1 = d.n1, na = d.na, nj = c.nj;
    int r1a = blockIdx.y * kCvjR1, r1b = min(n1, r1a + kCvjR1);     // this CTA's r1 chunk
    int w = d.blk_wave[g], el = d.blk_elec[g], om = d.blk_om[g];
    double *fr = cvsm;                       // [na][kCvjR1] psi / sqrt(ah2) of this CTA's r1 chunk
    double *dj = cvsm + (size_t)na * kCvjR1; // [nj][na]
    const int *m = c.r2abs + (size_t)w * na * n1;
    int cw = r1b - r1a;
    for (int e = threadIdx.x; e < na * cw; e += blockDim.x) {
        int a = e / cw, ir1 = r1a + e % cw;
        int ir = m[(size_t)a * n1 + ir1];
        fr[(size_t)a * kCvjR1 + (ir1 - r1a)] = (ir >= 0) ? c.psi[d.foff[(size_t)g * na + a] + ir] / c.sah2 : 0.0;
    }
    for (int e = threadIdx.x; e < nj * na; e += blockDim.x) {
        int jj = e / na, a = e % na;
        int j = c.jini + jj;
        dj[e] = cvj_on(c, g, j)
                    ? c.djall[c.djoff[w] + (((size_t)om * d.ne + (el - 1)) * (c.wnangu2[w] + 1) + j) * na + a]
                    : 0.0;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < cw * nj; e += blockDim.x) {
        int ir1 = r1a + e / nj, jj = e % nj;
        double xj = 0.0;
        for (int ia = 0; ia < na; ia++) {
            int a = na - 1 - ia;                  // angle order of the flat vector
            xj = xj + fr[(size_t)a * kCvjR1 + (ir1 - r1a)] * dj[(size_t)jj * na + a];
        }
        c.xj[((size_t)g * n1 + ir1) * nj + jj] = xj;
    }
}

// 2. Cvj(g, j, v) = sum_r1 xj(g, r1, j) fd(r1, v, j); one warp per (g, j, v)
__global__ void __launch_bounds__(256) k_cvj_fd(DevGrid d, CvjArgs c)
{
    int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    int nj = c.nj, nv = c.nv, n1 = d.n1;
    if (wid >= d.G * nj * nv) return;
    int g = wid / (nj * nv), jv = wid % (nj * nv), jj = jv / nv, iv = jv % nv;
    int j = c.jini + jj, el = d.blk_elec[g];
    int nob = c.nobc[(size_t)(el - 1) * nj + jj];
    int maxnv = c.nvmax < nob ? c.nvmax : nob;
    bool on = cvj_on(c, g, j) && c.nvini + iv <= maxnv;
    double r = 0.0;
    if (on) {
        const double *f = c.fd + (((size_t)(el - 1) * nj + jj) * nv + iv) * n1;
        const double *x = c.xj + (size_t)g * n1 * nj + jj;
        for (int ir1 = lane; ir1 < n1; ir1 += 32) r += x[(size_t)ir1 * nj] * f[ir1];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    if (lane == 0) c.cvj[((size_t)g * nj + jj) * nv + iv] = on ? r : 0.0;
}

// Mixed path, 1 and 2 in FP32: the projection reads the FP32 copy of psi and the
// FP32 Djmmp columns (0 where Cvj is off), Cvj goes to this iteration's ring slot
// (0 for the gated elastic channel) and, as FP64, to cvj
__global__ void __launch_bounds__(256) k_cvj_proj32(DevGrid d, CvjArgs c)
{
    extern __shared__ float cvs[];
    const int g = blockIdx.x, n1 = d.n1, na = d.na, nj = c.nj;
    const int r1a = blockIdx.y * kCvjR1, r1b = min(n1, r1a + kCvjR1), cw = r1b - r1a;
    const int w = d.blk_wave[g];
    float *fr = cvs;                          // [na][kCvjR1]
    float *dj = cvs + (size_t)na * kCvjR1;    // [nj][na]
    const int *m = c.r2abs + (size_t)w * na * n1;
    for (int e = threadIdx.x; e < na * cw; e += blockDim.x) {
        int a = e / cw, i = e % cw;
        int ir = m[(size_t)a * n1 + r1a + i];
        fr[a * kCvjR1 + i] = (ir >= 0) ? c.pk32[d.foff[(size_t)g * na + a] + ir] * c.rsah2f : 0.f;
    }
    for (int e = threadIdx.x; e < nj * na; e += blockDim.x) dj[e] = c.dj32[(size_t)g * nj * na + e];
    __syncthreads();
    for (int e = threadIdx.x; e < cw * nj; e += blockDim.x) {
        int i = e / nj, jj = e % nj;
        float xj = 0.f;
        for (int ia = 0; ia < na; ia++) {
            int a = na - 1 - ia;                  // angle order of the flat vector
            xj = fmaf(fr[a * kCvjR1 + i], dj[jj * na + a], xj);
        }
        c.xj32[((size_t)g * n1 + r1a + i) * nj + jj] = xj;
    }
}

__global__ void __launch_bounds__(256) k_cvj_fd32(DevGrid d, CvjArgs c)
{
    int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    int nj = c.nj, nv = c.nv, n1 = d.n1;
    if (wid >= d.G * nj * nv) return;
    int g = wid / (nj * nv), jv = wid % (nj * nv), jj = jv / nv, iv = jv % nv;
    int j = c.jini + jj, el = d.blk_elec[g];
    int nob = c.nobc[(size_t)(el - 1) * nj + jj];
    int maxnv = c.nvmax < nob ? c.nvmax : nob;
    bool on = cvj_on(c, g, j) && c.nvini + iv <= maxnv;
    float r = 0.f;
    if (on) {
        const float *f = c.fd32 + (((size_t)(el - 1) * nj + jj) * nv + iv) * n1;
        const float *x = c.xj32 + (size_t)g * n1 * nj + jj;
        for (int ir1 = lane; ir1 < n1; ir1 += 32) r = fmaf(x[(size_t)ir1 * nj], f[ir1], r);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    if (lane == 0) {
        const bool gated = c.gate && c.blk_isref[g] && j == c.jref && c.nvini + iv == c.nvref;
        c.cvj[wid] = on ? (double)r : 0.0;
        c.ring[wid] = (on && !gated) ? r : 0.f;
    }
}

// the FP32 Djmmp columns of the projection: dj32[g][jj][a], 0 where Cvj is off
__global__ void k_cvj_dj32(DevGrid d, CvjArgs c, float *__restrict__ dj32)
{
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int na = d.na, nj = c.nj;
    if (e >= (int64_t)d.G * nj * na) return;
    int a = (int)(e % na), jj = (int)((e / na) % nj), g = (int)(e / ((int64_t)na * nj));
    int w = d.blk_wave[g], el = d.blk_elec[g], om = d.blk_om[g], j = c.jini + jj;
    dj32[e] =
        cvj_on(c, g, j)
            ? (float)c.djall[c.djoff[w] + (((size_t)om * d.ne + (el - 1)) * (c.wnangu2[w] + 1) + j) * na + a]
            : 0.f;
}

// zS2(E, row) += sum_s Cvj_s(row) C_s(E) over the ring slots: FP32 products and
// sums (a 64 x 64 (E, row) tile per CTA, 4 x 4 per thread), added once to the
// FP64 accumulators, so zS2 is read and written once per flush instead of once
// per iteration
constexpr int kCvFlushR = 64, kCvFlushE = 64;
__global__ void __launch_bounds__(256) k_cvj_flush(const float *__restrict__ ring, const float *__restrict__ cring,
                                                   unsigned slot_mask, int R, int netot, double *__restrict__ zs2)
{
    __shared__ float sc[kFluxRing][kCvFlushE][2];
    __shared__ float sr[kFluxRing][kCvFlushR];
    const int r0 = blockIdx.x * kCvFlushR, e0 = blockIdx.y * kCvFlushE;
    for (int i = threadIdx.x; i < kFluxRing * kCvFlushE * 2; i += blockDim.x) {
        int s = i / (kCvFlushE * 2), q = i % (kCvFlushE * 2);
        int e = e0 + q / 2;
        sc[s][q / 2][q & 1] =
            (e < netot && ((slot_mask >> s) & 1u)) ? cring[((size_t)s * netot + e) * 2 + (q & 1)] : 0.f;
    }
    for (int i = threadIdx.x; i < kFluxRing * kCvFlushR; i += blockDim.x) {
        int s = i / kCvFlushR, q = i % kCvFlushR;
        int row = r0 + q;
        sr[s][q] = row < R ? ring[(size_t)s * R + row] : 0.f;
    }
    __syncthreads();
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;   // E = e0 + tx + 16 i, row = r0 + ty + 16 j
    float ar[4][4], ai[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) ar[i][j] = ai[i][j] = 0.f;
    for (int s = 0; s < kFluxRing; s++) {
        float cr[4], ci[4], v[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            cr[i] = sc[s][tx + 16 * i][0];
            ci[i] = sc[s][tx + 16 * i][1];
        }
#pragma unroll
        for (int j = 0; j < 4; j++) v[j] = sr[s][ty + 16 * j];
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) {
                ar[i][j] = fmaf(v[j], cr[i], ar[i][j]);
                ai[i][j] = fmaf(v[j], ci[i], ai[i][j]);
            }
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int row = r0 + ty + 16 * j;
        if (row >= R) continue;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int e = e0 + tx + 16 * i;
            if (e >= netot) continue;
            double2 *z = reinterpret_cast<double2 *>(zs2 + ((size_t)row * netot + e) * 2);
            double2 a = *z;
            a.x += (double)ar[i][j];
            a.y += (double)ai[i][j];
            *z = a;
        }
    }
}

// 3. zS2(E, v, j, g) += Cvj C_k(E), the elastic reference channel gated below kminelastic
__global__ void __launch_bounds__(256) k_cvj_acc(DevGrid d, CvjArgs c)
{
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int nj = c.nj, nv = c.nv, netot = c.netot;
    if (e >= (int64_t)d.G * nj * nv * netot) return;
    int ie = (int)(e % netot);
    int64_t r = e / netot;
    int iv = (int)(r % nv);
    int jj = (int)((r / nv) % nj);
    int g = (int)(r / ((int64_t)nv * nj));
    int j = c.jini + jj, el = d.blk_elec[g];
    int nob = c.nobc[(size_t)(el - 1) * nj + jj];
    int maxnv = c.nvmax < nob ? c.nvmax : nob;
    if (!(cvj_on(c, g, j) && c.nvini + iv <= maxnv)) return;
    if (c.gate && c.blk_isref[g] && j == c.jref && c.nvini + iv == c.nvref) return;
    double z = c.cvj[r];
    c.zs2[2 * e] += z * c.zck[2 * ie];
    c.zs2[2 * e + 1] += z * c.zck[2 * ie + 1];
}

// totalflux (mod_flux_01y2.f:778-816) for one wave's flux points
__global__ void k_totalflux(const double *__restrict__ zcr, const double *__restrict__ zcdr,
                            const int *__restrict__ fblock, const int *__restrict__ nelebas, int nflux, int netot,
                            int nelec, const double *__restrict__ reacfct, double ah1, double *__restrict__ out,
                            double *__restrict__ outelec)
{
    int ie = blockIdx.x * blockDim.x + threadIdx.x;
    if (ie >= netot) return;
    double s = 0.0;
    double se[8];
    for (int e = 0; e < 8; e++) se[e] = 0.0;
    for (int f = 0; f < nflux; f++) {
        size_t o = ((size_t)f * netot + ie) * 2;
        double im = zcr[o] * zcdr[o + 1] + (-zcr[o + 1]) * zcdr[o];
        s = s + im;
        int el = nelebas[fblock[f]] - 1;
        if (el < 8) se[el] = se[el] + im;
    }
    out[ie] = s * reacfct[ie] / ah1;
    if (outelec)
        for (int e = 0; e < nelec && e < 8; e++) outelec[(size_t)e * netot + ie] = se[e] * reacfct[ie] / ah1;
}

// ---------------------------------------------------------------------------
// set-up: explicit angle x angle kinetic matrices from Djmmp and the scalars
// (angkinj2 :255-272 and bfgridl2mat :419-468 assembled on the device)
// ---------------------------------------------------------------------------
struct KinBuildArgs {
    int na, n1, n2, ne;
    const int *blk_wave, *blk_elec, *blk_om, *blk_local;
    const int *wnojb;            // [G] nojbas
    const int *wjbas;            // [G][na]
    const double *yj2;           // [G][n1][na]
    const double *djmmp;         // all waves concatenated
    const int64_t *djoff;        // [W]
    const int *wnangu2, *wj0, *winc, *wiommin, *wiommax, *wnom, *wnj2;   // [W]
    const double *l2tab;         // all waves
    const int64_t *l2off;        // [W]
    const char *l2used;
    const int64_t *l2uoff;       // [W]
};

__device__ inline double djget(const KinBuildArgs &k, int w, int iom, int ielec, int j, int a)
{
    return k.djmmp[k.djoff[w] + (((size_t)iom * k.ne + (ielec - 1)) * (k.wnangu2[w] + 1) + j) * k.na + a];
}

// xj2[ir1][i][j] = sum_k yj2[ir1][k] D_g(i, j_k) D_g(j, j_k) with block g's basis and
// Djmmp: the block's own j^2 matrix, or a channel-pair matrix of the electronic
// Coriolis variant with g its source channel (yj2 then holds the pair's scalars)
template <typename T>
__global__ void k_build_xj2(KinBuildArgs k, const double *__restrict__ yj2, T *__restrict__ xj2, int g)
{
    int na = k.na;
    int ir1 = blockIdx.x;
    int w = k.blk_wave[g], e = k.blk_elec[g], om = k.blk_om[g];
    const double *yy = yj2 + (size_t)ir1 * na;
    for (int ij = threadIdx.x; ij < na * na; ij += blockDim.x) {
        int i = ij / na, j = ij % na;
        double acc = 0.0;
        for (int q = 0; q < k.wnojb[g]; q++) {
            int jb = k.wjbas[(size_t)g * na + q];
            double x1 = djget(k, w, om, e, jb, i), x2 = djget(k, w, om, e, jb, j);
            acc = __dadd_rn(acc, __dmul_rn(__dmul_rn(yy[q], x1), x2));
        }
        xj2[(size_t)ir1 * na * na + ij] = (T)acc;
    }
}

template <typename T>
__global__ void k_build_xl2p(KinBuildArgs k, T *__restrict__ xl2p, int s, int slot)
{
    int na = k.na;
    int ir2 = blockIdx.x;
    int w = k.blk_wave[s], e = k.blk_elec[s], oms = k.blk_om[s];
    int q = slot - 1;
    int omt = oms - q;
    int iommin = k.wiommin[w], iommax = k.wiommax[w], nom = k.wnom[w], nj2 = k.wnj2[w];
    T *out = xl2p + (((size_t)s * 3 + slot) * k.n2 + ir2) * na * na;
    bool ok = (omt >= iommin && omt <= iommax);
    for (int ij = threadIdx.x; ij < na * na; ij += blockDim.x) {
        int i = ij / na, j = ij % na;
        double acc = 0.0;
        if (ok)
            for (int jidx = 0; jidx < nj2; jidx++) {
                int jv = k.wj0[w] + jidx * k.winc[w];
                if (jv > (na - 1) * k.winc[w]) break;
                size_t u = (((size_t)(e - 1) * nj2 + jidx) * nom + (omt - iommin)) * nom + (oms - iommin);
                if (!k.l2used[k.l2uoff[w] + u]) continue;
                double yyy = k.l2tab[k.l2off[w] + ((((size_t)(e - 1) * nj2 + jidx) * k.n2 + ir2) * nom + (omt - iommin)) * nom + (oms - iommin)];
                double x11 = djget(k, w, omt, e, jv, i), x22 = djget(k, w, oms, e, jv, j);
                acc = __dadd_rn(acc, __dmul_rn(__dmul_rn(x11, x22), yyy));
            }
        out[ij] = (T)acc;
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
template <typename T>
void launch_scatter(Ctx &c, const double *psi, float *psi32, int g_begin, int g_end)
{
    int nseg = (g_end - g_begin) * c.na;
    if (nseg <= 0) return;
    unsigned *xmax = sizeof(T) == 4 ? c.d_xmax : nullptr;
    // the scattered rectangle replaces whatever the update left: its slabs' largest
    // |X| start from zero, so a restart scales X exactly as the uninterrupted run
    if (xmax) cudaMemsetAsync(xmax + (size_t)g_begin * c.na, 0, (size_t)nseg * sizeof(unsigned), c.stream);
    k_scatter<T><<<dim3(nseg, c.nchunk), 256, 0, c.stream>>>(devgrid(c), (T *)c.d_X, psi, psi32, g_begin * c.na,
                                                              xmax);
    LAUNCH_CHECK(c);
}

static size_t col_smem(Ctx &c, size_t tsz) { return tsz * (size_t)c.n1 * (COL_W + COL_KC); }
static size_t ang_desc(Ctx &c) { return (size_t)c.na * c.ang_cw * 16 + 16; }
static size_t angj_smem(Ctx &c, size_t tsz)
{
    return tsz * ((size_t)c.na * c.ang_cw + (size_t)c.na * (c.na + 1)) + ang_desc(c);
}
static size_t angl_smem(Ctx &c, size_t tsz)
{
    return tsz * ((size_t)c.na * c.ang_cw + (size_t)c.na * c.ang_cw + (size_t)c.na * (c.na + 1)) + ang_desc(c);
}

// the electronic Coriolis targets among blocks [g_begin, g_end)
template <typename T, typename HT>
static void launch_ecor(Ctx &c, const DevGrid &d, const T *X, HT *H, int g_begin, int g_end)
{
    if (c.ec_nt == 0 || !c.d_xj2e || c.na <= 1) return;
    const long lo = std::lower_bound(c.h_ec_tgt.begin(), c.h_ec_tgt.end(), g_begin) - c.h_ec_tgt.begin();
    const long hi = std::lower_bound(c.h_ec_tgt.begin(), c.h_ec_tgt.end(), g_end) - c.h_ec_tgt.begin();
    if (hi <= lo) return;
    dim3 grid(c.ncj, c.n1, (unsigned)(hi - lo));
    k_ang_je<T, HT><<<grid, 256, angl_smem(c, sizeof(T)), c.stream>>>(
        d, X, (const T *)c.d_xj2e, H, c.d_tj_ptr, c.d_tj, c.ncj, c.d_ec_tgt + lo, c.d_ec_src + lo * c.ec_slots,
        c.d_ec_mat + lo * c.ec_slots, c.ec_slots, c.ang_cw);
    LAUNCH_CHECK(c);
}

template <typename T>
void launch_hphi(Ctx &c, const double *psi, int g_begin, int g_end)
{
    int ng = g_end - g_begin;
    if (ng <= 0) return;
    DevGrid d = devgrid(c);
    constexpr int BM = RowCfg<T>::BM, BN = RowCfg<T>::BN;
    int64_t row0 = (int64_t)g_begin * c.na * c.n1;
    int64_t nrows = (int64_t)ng * c.na * c.n1;
    dim3 gr((unsigned)((nrows + BM - 1) / BM), ((c.n2 + 1) / 2 + BN - 1) / BN);   // folded: ceil(n2/2) columns
    if (sizeof(T) == 4 && c.use_tc_dst2d) {
        // mixed path: the whole DST chain of each slab in one tensor-core kernel, H in FP32
        stage_mark(c, 0);
        launch_tc_dst2d(c, (const float *)c.d_X, c.d_h32, g_begin, g_end);
        stage_mark(c, 1);
        stage_mark(c, 2);
        k_quirk<float><<<ng * c.na, 128, 0, c.stream>>>(d, psi, c.d_h32, c.d_quirk_ptr, c.d_quirk, g_begin * c.na);
        LAUNCH_CHECK(c);
        stage_mark(c, 3);
        if (c.use_tc_ang) {
            launch_tc_ang(c, (const float *)c.d_X, c.d_h32, g_begin, g_end, c.x_t);
            launch_ecor<float, float>(c, d, (const float *)c.d_X, c.d_h32, g_begin, g_end);
            stage_mark(c, 4);
            return;
        }
        // the explicit angular kernels accumulate in FP64: widen H first
        k_h32_to_h<<<dim3(ng * c.na, c.nchunk), 256, 0, c.stream>>>(d, c.d_h32, c.d_h, g_begin * c.na);
        LAUNCH_CHECK(c);
    } else if (sizeof(T) == 4 && tc_dst_supported(c)) {
        // mixed path: the three DST passes on the tensor cores
        launch_tc_dst(c, (const float *)c.d_X, (float *)c.d_Y, c.d_h, g_begin, g_end, 0);
    } else {
        // 1. DST along R
        stage_mark(c, 0);
        const bool rader = sizeof(T) == 8 && c.d_rd_tw;
        if (rader)
            k_dst_rows_rader<false><<<rd_grid(), 256, 0, c.stream>>>(d, (const double *)c.d_X, (double *)c.d_Y,
                                                                     nullptr, rd_tab(c), g_begin * c.na, ng * c.na);
        else
            k_dst_rows<T, false><<<gr, 256, 0, c.stream>>>(d, (const T *)c.d_X, (const T *)c.d_S2, (T *)c.d_Y,
                                                            nullptr, c.d_nopr1, row0, nrows);
        LAUNCH_CHECK(c);
        // 2. DST along r, k-space scaling, DST along r
        stage_mark(c, 1);
        dim3 gc(ng * c.na, (c.n2 + COL_W - 1) / COL_W);
        k_dst_cols<T><<<gc, 256, col_smem(c, sizeof(T)), c.stream>>>(d, (T *)c.d_Y, (const T *)c.d_S1, c.d_S1off,
                                                                      c.d_nopr1, c.d_p2r1, c.d_p2r2, c.grid.radcutmax,
                                                                      g_begin * c.na);
        LAUNCH_CHECK(c);
        // 3. DST along R, gathered into H at the stored points
        stage_mark(c, 2);
        if (rader)
            k_dst_rows_rader<true><<<rd_grid(), 256, 0, c.stream>>>(d, (const double *)c.d_Y, nullptr, c.d_h,
                                                                    rd_tab(c), g_begin * c.na, ng * c.na);
        else
            k_dst_rows<T, true><<<gr, 256, 0, c.stream>>>(d, (const T *)c.d_Y, (const T *)c.d_S2, nullptr, c.d_h,
                                                           c.d_nopr1, row0, nrows);
        LAUNCH_CHECK(c);
    }
    // points beyond the r1 DST length keep psi
    if (!(sizeof(T) == 4 && c.use_tc_dst2d)) {
        k_quirk<double><<<ng * c.na, 128, 0, c.stream>>>(d, psi, c.d_h, c.d_quirk_ptr, c.d_quirk, g_begin * c.na);
        LAUNCH_CHECK(c);
        stage_mark(c, 3);
    }
    // 4. angular kinetic terms
    if (sizeof(T) == 4 && c.use_tc_ang) {
        // mixed path: j^2 + l^2 + Coriolis in one factorised tensor-core contraction
        launch_tc_ang(c, (const float *)c.d_X, c.d_h, g_begin, g_end, c.x_t);
        stage_mark(c, 4);
    } else if (c.na > 1) {
        dim3 gj(c.ncj, c.n1, ng);
        k_ang_j<T><<<gj, 256, angj_smem(c, sizeof(T)), c.stream>>>(d, (const T *)c.d_X, (const T *)c.d_xj2, c.d_h,
                                                                    c.d_tj_ptr, c.d_tj, c.ncj, g_begin, c.ang_cw);
        LAUNCH_CHECK(c);
        stage_mark(c, 4);
        dim3 gl(c.ncl, c.n2, ng);
        k_ang_l<T><<<gl, 256, angl_smem(c, sizeof(T)), c.stream>>>(d, (const T *)c.d_X, (const T *)c.d_xl2p, c.d_h,
                                                                    c.d_tl_ptr, c.d_tl, c.d_cpl, c.ncl, g_begin, c.ang_cw);
        LAUNCH_CHECK(c);
    }
    launch_ecor<T, double>(c, d, (const T *)c.d_X, c.d_h, g_begin, g_end);
}

template <typename T>
void launch_update(Ctx &c, int first)
{
    UpdArgs u;
    u.xmax = sizeof(T) == 4 ? c.d_xmax : nullptr;
    u.H = c.d_h;
    u.pk = c.d_pk;
    u.pkm1 = c.d_pkm1;
    u.out = c.d_pkm1;
    u.vsrc = c.d_vsrc;
    u.absfr1 = c.d_absfr1;
    u.absfr2 = c.d_absfr2;
    u.absfr1f = c.d_absfr1f;
    u.abs_start = c.d_abs_start;
    u.absfr2f = c.d_absfr2f;
    u.emindlt = c.grid.emindlt;
    u.delta2 = c.grid.delta2;
    u.rdelta = 1.0 / c.grid.delta2;
    u.r2delta = 2.0 / c.grid.delta2;
    u.vr32 = c.d_vr32;
    u.pk32 = c.d_pk32;
    u.out32 = c.d_pkm1_32;
    u.r2df = (float)(2.0 / c.grid.delta2);
    u.desc = c.d_upd_desc;
    u.nchunk = c.nchunk;
    u.first = first;
    u.normpart = c.d_normpart;
    u.nofe = c.nofemax;
    u.zcke = c.d_zcke;
    u.zfe = c.d_zfe_ptrs;
    u.wflat0 = c.d_wflat0;
    stage_mark(c, 5);
    if (c.h32) {
        u.H = c.d_h32;
        k_update<T, float><<<c.n_upd_chunks, 256, 0, c.stream>>>(devgrid(c), u, (T *)c.d_X);
    } else {
        k_update<T, double><<<c.n_upd_chunks, 256, 0, c.stream>>>(devgrid(c), u, (T *)c.d_X);
    }
    LAUNCH_CHECK(c);
}

template <typename T>
void launch_build_kinetic(Ctx &c)
{
    KinBuildArgs k;
    k.na = c.na; k.n1 = c.n1; k.n2 = c.n2; k.ne = c.ne;
    k.blk_wave = c.d_blk_wave; k.blk_elec = c.d_blk_elec; k.blk_om = c.d_blk_om; k.blk_local = nullptr;
    k.wnojb = c.d_blk_nojb; k.wjbas = c.d_blk_jbas; k.yj2 = c.d_blk_yj2;
    k.djmmp = c.d_djall; k.djoff = c.d_djoff;
    k.wnangu2 = c.d_wnangu2; k.wj0 = c.d_wj0; k.winc = c.d_winc; k.wiommin = c.d_wiommin;
    k.wiommax = c.d_wiommax; k.wnom = c.d_wnom; k.wnj2 = c.d_wnj2;
    k.l2tab = c.d_l2all; k.l2off = c.d_l2off; k.l2used = c.d_l2used; k.l2uoff = c.d_l2uoff;
    const size_t mat = (size_t)c.n1 * c.na * c.na;
    for (int p = 0; p < c.ec_pairs && c.d_xj2e; p++) {
        k_build_xj2<T><<<c.n1, 256, 0, c.stream>>>(k, c.d_ec_y + (size_t)p * c.n1 * c.na, (T *)c.d_xj2e + p * mat,
                                                    c.h_ec_psrc[p]);
        LAUNCH_CHECK(c);
    }
    if (!c.d_xj2) return;
    for (int g = 0; g < c.G; g++) {
        k_build_xj2<T><<<c.n1, 256, 0, c.stream>>>(k, c.d_blk_yj2 + (size_t)g * c.n1 * c.na, (T *)c.d_xj2 + g * mat,
                                                    g);
        LAUNCH_CHECK(c);
        for (int slot = 0; slot < 3; slot++) {
            if (!c.h_slot_used[(size_t)g * 3 + slot]) continue;
            k_build_xl2p<T><<<c.n2, 256, 0, c.stream>>>(k, (T *)c.d_xl2p, g, slot);
            LAUNCH_CHECK(c);
        }
    }
}

void set_kernel_attributes(Ctx &c)
{
    cudaFuncSetAttribute(k_cvj_proj, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_dst_cols<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)col_smem(c, 8));
    cudaFuncSetAttribute(k_dst_cols<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)col_smem(c, 4));
    cudaFuncSetAttribute(k_ang_j<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)angj_smem(c, 8));
    cudaFuncSetAttribute(k_ang_j<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)angj_smem(c, 4));
    cudaFuncSetAttribute(k_ang_l<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)angl_smem(c, 8));
    cudaFuncSetAttribute(k_ang_l<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)angl_smem(c, 4));
    cudaFuncSetAttribute(k_ang_je<double, double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)angl_smem(c, 8));
    cudaFuncSetAttribute(k_ang_je<float, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)angl_smem(c, 4));
    cudaFuncSetAttribute(k_ang_je<float, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)angl_smem(c, 4));
}

bool fit_smem(Ctx &c, size_t optin)
{
    // the widest angular column chunk whose staged matrices fit (FP64 sizes)
    for (int cw = 64; cw >= 8; cw /= 2) {
        c.ang_cw = cw;
        size_t m = col_smem(c, 8);
        if (angj_smem(c, 8) > m) m = angj_smem(c, 8);
        if (angl_smem(c, 8) > m) m = angl_smem(c, 8);
        if (m <= optin) return true;
    }
    return false;
}

// accumulators of iteration it for every wave (CoefEcheby, totalflux_k, Cvjflux_k, funE coefficients)
static CvjArgs cvj_args(Ctx &c, bool gate)
{
    CvjArgs a;
    a.psi = c.d_pk;
    a.r2abs = c.d_r2abs;
    a.djall = c.d_djall;
    a.djoff = c.d_djoff;
    a.wnangu2 = c.d_wnangu2;
    a.blk_j00 = c.d_blk_j00;
    a.blk_inc = c.d_blk_inc;
    a.blk_isref = c.d_blk_isref;
    a.fd = c.d_fd;
    a.nobc = c.d_nobc;
    a.xj = c.d_xj;
    a.cvj = c.d_cvj;
    a.zs2 = c.d_zs2;
    a.zck = c.d_zck;
    a.jini = c.jini; a.jmax = c.jmax; a.nvini = c.nvini; a.nvmax = c.nvmax;
    a.nj = c.nj; a.nv = c.nv; a.netot = c.netot; a.jref = c.jref; a.nvref = c.nvref;
    a.gate = gate ? 1 : 0;
    a.sah2 = c.sah2;
    a.pk32 = c.d_pk32;
    a.dj32 = c.d_dj32;
    a.fd32 = c.d_fd32;
    a.xj32 = c.d_xj32;
    a.ring = nullptr;
    a.rsah2f = (float)(1.0 / c.sah2);
    return a;
}

// C_k(E) at funE's energies for iteration it, before the update kernel adds
// C_k(E) psi_k to zfe (funE follows the update, main_madwave3.f:350-352)
void launch_fe_coef(Ctx &c, int64_t it)
{
    const int64_t itarg = c.capturing ? it - c.cap_it0 : it;
    const int64_t *bp = c.capturing ? c.d_itbase : nullptr;
    for (size_t w = 0; w < c.waves.size(); w++) {
        WaveTables &t = c.waves[w];
        if (t.nofe > 0) {
            k_coefecheby<<<(t.nofe + 127) / 128, 128, 0, c.stream>>>(c.wdev[w].efe, t.nofe, c.grid.emindlt,
                                                                     c.grid.delta2, c.grid.hbr,
                                                                     itarg, c.d_zcke + (size_t)w * c.nofemax * 2,
                                                                     nullptr, 0, nullptr, bp);
            LAUNCH_CHECK(c);
        }
    }
}

void launch_accumulators(Ctx &c, int64_t it)
{
    stage_mark(c, 6);
    DevGrid d = devgrid(c);
    const bool ring = c.d_fring != nullptr;
    const int64_t itarg = c.capturing ? it - c.cap_it0 : it;
    const int64_t *bp = c.capturing ? c.d_itbase : nullptr;
    bool gate = c.gate_elastic && it < c.kminelastic;
    const bool flux_on = c.NF > 0 && !(gate && c.waves[0].iprod == 1);
    k_coefecheby<<<(c.netot + 127) / 128, 128, 0, c.stream>>>(
        c.d_etot, c.netot, c.grid.emindlt, c.grid.delta2, c.grid.hbr, itarg, c.d_zck, ring ? c.d_cring : nullptr,
        flux_on ? 0 : 1, c.d_cvcring ? c.d_cvcring + (size_t)(it % kFluxRing) * c.netot * 2 : nullptr, bp);
    LAUNCH_CHECK(c);
    if (ring) {
        if (flux_on) {
            k_flux_deriv<<<(c.NF * 32 + 255) / 256, 256, 0, c.stream>>>(
                c.d_pk, c.d_fl_idx, c.d_fl_dptr, c.d_fl_didx, c.d_fl_dir1, c.d_zar, c.NF, c.d_fpsi, c.d_fring,
                c.d_pk32, c.d_zar32, c.fl_runs ? c.d_fl_rptr : nullptr, c.fl_runs ? c.d_fl_runs : nullptr, itarg, bp);
            LAUNCH_CHECK(c);
        }
        // a slice every fl_q iterations, also while the flux is gated (its C slot is 0 then)
        if (it % c.fl_q == c.fl_q - 1) {
            const int P = kFluxSlots / c.fl_q, chunk = (c.NF + P - 1) / P;
            dim3 g((chunk + kFlushF - 1) / kFlushF, (c.netot + kFlushE - 1) / kFlushE);
            k_flux_flush<<<g, 256, 0, c.stream>>>(c.d_fring, c.d_cring, c.d_fl_poti, c.d_etot, c.netot, c.NF, chunk,
                                                  c.fl_q, itarg, bp, 0, c.d_zcr, c.d_zcdr);
            LAUNCH_CHECK(c);
        }
    } else if (flux_on) {
        k_flux_deriv<<<(c.NF * 32 + 255) / 256, 256, 0, c.stream>>>(
            c.d_pk, c.d_fl_idx, c.d_fl_dptr, c.d_fl_didx, c.d_fl_dir1, c.d_zar, c.NF, c.d_fpsi, nullptr, c.d_pk32,
            c.d_zar32, nullptr, nullptr, itarg, bp);
        LAUNCH_CHECK(c);
        {
            dim3 g((c.NF + kFluxPerBlock - 1) / kFluxPerBlock, (c.netot + 127) / 128);
            k_flux_acc<<<g, 128, 0, c.stream>>>(c.d_fpsi, c.d_fl_poti, c.d_etot, c.d_zck, c.netot, c.NF, c.d_zcr,
                                                c.d_zcdr);
            LAUNCH_CHECK(c);
        }
    }
    if (c.n2 > 1 && c.d_cvring) {
        // mixed path: FP32 projection, Cvj into the ring, zS2 at the flush
        CvjArgs a = cvj_args(c, gate);
        a.ring = c.d_cvring + (size_t)(it % kFluxRing) * c.G * c.nj * c.nv;
        size_t sm32 = sizeof(float) * ((size_t)c.na * kCvjR1 + (size_t)c.nj * c.na);
        k_cvj_proj32<<<dim3(c.G, (c.n1 + kCvjR1 - 1) / kCvjR1), 256, sm32, c.stream>>>(d, a);
        LAUNCH_CHECK(c);
        k_cvj_fd32<<<(c.G * c.nj * c.nv * 32 + 255) / 256, 256, 0, c.stream>>>(d, a);
        LAUNCH_CHECK(c);
        if (it % kFluxRing == kFluxRing - 1) {   // the ring's 32 iterations into zS2
            const int R = c.G * c.nj * c.nv;
            dim3 g((R + kCvFlushR - 1) / kCvFlushR, (c.netot + kCvFlushE - 1) / kCvFlushE);
            k_cvj_flush<<<g, 256, 0, c.stream>>>(c.d_cvring, c.d_cvcring, 0xffffffffu, R, c.netot, c.d_zs2);
            LAUNCH_CHECK(c);
        }
    } else if (c.n2 > 1) {
        CvjArgs a = cvj_args(c, gate);
        size_t smp = sizeof(double) * ((size_t)c.na * kCvjR1 + (size_t)c.nj * c.na);
        k_cvj_proj<<<dim3(c.G, (c.n1 + kCvjR1 - 1) / kCvjR1), 256, smp, c.stream>>>(d, a);
        LAUNCH_CHECK(c);
        k_cvj_fd<<<(c.G * c.nj * c.nv * 32 + 255) / 256, 256, 0, c.stream>>>(d, a);
        LAUNCH_CHECK(c);
        int64_t tot = (int64_t)c.G * c.nj * c.nv * c.netot;
        k_cvj_acc<<<(unsigned)((tot + 255) / 256), 256, 0, c.stream>>>(d, a);
        LAUNCH_CHECK(c);
    }
    // prodpaq + prodcvj (main_madwave3.f:346-349), after Cvjflux_k
    if (c.n1 > 1 && c.n2 > 1) launch_product(c);
}

// ---------------------------------------------------------------------------
// Product-state projection (iprod = 2), mod_coortrans01_02.f:694-825
// ---------------------------------------------------------------------------
// prodpaq, step 1: funprod(R, angle, block) = sum of transRgjac psi over the
// stored points of (block, angle) at R, in the points' order; one thread per bin
__global__ void __launch_bounds__(256) k_prod_bins(const double *__restrict__ psi, const int *__restrict__ bin_ptr,
                                                   const int64_t *__restrict__ bin_idx,
                                                   const double *__restrict__ bin_w, int nbins,
                                                   double *__restrict__ fun)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nbins) return;
    double s = 0.0;
    for (int k = bin_ptr[b]; k < bin_ptr[b + 1]; k++) s = s + bin_w[k] * psi[bin_idx[k]];
    fun[b] = s;
}

// prodpaq, step 2: Cvjprod(v, j, Omega) = sum over blocks and (angle, R) of
// prodwf(R, angle, e, v, j, Omega) (funprod dtrans(R, angle, Omega, block)); one
// warp per (Omega, j, v), 0 outside j >= max(jiniprod, Omega), v <= noBCprod(j)
__global__ void __launch_bounds__(256) k_prod_proj(const double *__restrict__ fun, const double *__restrict__ dtrans,
                                                   const double *__restrict__ prodwf,
                                                   const int *__restrict__ nobcprod,
                                                   const int *__restrict__ blk_elec, int ncan, int nelec, int K,
                                                   int om0, int nom, int jp0, int njp, int vp0, int nvp,
                                                   double *__restrict__ cvjprod)
{
    const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (row >= nom * njp * nvp) return;                 // whole warps
    const int o = row / (njp * nvp), jj = (row / nvp) % njp, vv = row % nvp;
    const bool on = jp0 + jj >= max(jp0, om0 + o) && vp0 + vv <= nobcprod[jj];
    double x = 0.0;
    if (on) {
        for (int b = 0; b < ncan; b++) {
            const double *wf = prodwf + ((((size_t)o * njp + jj) * nvp + vv) * nelec + (blk_elec[b] - 1)) * K;
            const double *dt = dtrans + ((size_t)b * nom + o) * K;
            const double *fb = fun + (size_t)b * K;
            for (int k = lane; k < K; k += 32) x += wf[k] * (fb[k] * dt[k]);
        }
#pragma unroll
        for (int m = 16; m >= 1; m >>= 1) x += __shfl_xor_sync(0xffffffffu, x, m);
    }
    if (lane == 0) cvjprod[row] = x;
}

// prodcvj: zS2prod(E, v, j, Omega) += Cvjprod C_k(E); one thread per (row, E)
__global__ void __launch_bounds__(256) k_prod_acc(const double *__restrict__ cvjprod, const double *__restrict__ zck,
                                                  const int *__restrict__ nobcprod, int om0, int jp0, int njp,
                                                  int vp0, int nvp, int nrow, int netot,
                                                  double *__restrict__ zs2prod)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)nrow * netot) return;
    const int row = (int)(t / netot), ie = (int)(t % netot);
    const int o = row / (njp * nvp), jj = (row / nvp) % njp, vv = row % nvp;
    if (jp0 + jj < max(jp0, om0 + o) || vp0 + vv > nobcprod[jj]) return;
    const double z = cvjprod[row];
    double2 *s = reinterpret_cast<double2 *>(zs2prod) + t;
    double2 a = *s;
    a.x = a.x + (z * zck[2 * ie] - 0.0 * zck[2 * ie + 1]);
    a.y = a.y + (z * zck[2 * ie + 1] + 0.0 * zck[2 * ie]);
    *s = a;
}

void launch_product(Ctx &c)
{
    for (size_t w = 0; w < c.wdev.size() && w < c.prodt.size(); w++) {
        const ProdTables &pt = c.prodt[w];
        if (!pt.on) continue;
        const ProdDev &d = c.wdev[w].prod;
        const int nom = pt.om1 - pt.om0 + 1, njp = pt.jp1 - pt.jp0 + 1, nvp = pt.vp1 - pt.vp0 + 1;
        const int K = (pt.a1 - pt.a0 + 1) * (pt.n2p1 - pt.n2p0 + 1);
        k_prod_bins<<<(d.nbins + 255) / 256, 256, 0, c.stream>>>(c.d_pk, d.bin_ptr, d.bin_idx, d.bin_w, d.nbins,
                                                                d.fun);
        LAUNCH_CHECK(c);
        k_prod_proj<<<(d.nrow * 32 + 255) / 256, 256, 0, c.stream>>>(d.fun, d.dtrans, d.prodwf, d.nobcprod,
                                                                    d.blk_elec, c.waves[w].ncan, c.ne, K, pt.om0,
                                                                    nom, pt.jp0, njp, pt.vp0, nvp, d.cvjprod);
        LAUNCH_CHECK(c);
        const int64_t n = (int64_t)d.nrow * c.netot;
        k_prod_acc<<<(unsigned)((n + 255) / 256), 256, 0, c.stream>>>(d.cvjprod, c.d_zck, d.nobcprod, pt.om0, pt.jp0,
                                                                      njp, pt.vp0, nvp, d.nrow, c.netot, d.zs2prod);
        LAUNCH_CHECK(c);
    }
}

void flush_cvj(Ctx &c)
{
    if (!c.d_cvring) return;
    // slot = iteration mod 32, flushed whole at the iterations = 31 mod 32: pending
    // are the (now + 1) mod 32 iterations since, the slots (now - s) mod 32 < n
    const int n = (int)((c.it + 1) % kFluxRing);
    unsigned mask = 0;
    for (int s = 0; s < kFluxRing; s++)
        if ((int)(((c.it - s) % kFluxRing + kFluxRing) % kFluxRing) < n) mask |= 1u << s;
    if (mask) {
        const int R = c.G * c.nj * c.nv;
        dim3 g((R + kCvFlushR - 1) / kCvFlushR, (c.netot + kCvFlushE - 1) / kCvFlushE);
        k_cvj_flush<<<g, 256, 0, c.stream>>>(c.d_cvring, c.d_cvcring, mask, R, c.netot, c.d_zs2);
        LAUNCH_CHECK(c);
    }
    // every pending iteration is in zS2 now: clear the C slots so no later flush adds them again
    cudaMemsetAsync(c.d_cvcring, 0, sizeof(float) * kFluxRing * c.netot * 2, c.stream);
}

void build_cvj32(Ctx &c)
{
    if (!c.d_dj32 || c.n2 <= 1) return;
    CvjArgs a = cvj_args(c, false);
    int64_t tot = (int64_t)c.G * c.nj * c.na;
    k_cvj_dj32<<<(unsigned)((tot + 255) / 256), 256, 0, c.stream>>>(devgrid(c), a, c.d_dj32);
    LAUNCH_CHECK(c);
}

void flush_flux(Ctx &c)
{
    if (!c.d_fring || c.NF == 0) return;
    const int P = kFluxSlots / c.fl_q, chunk = (c.NF + P - 1) / P;
    dim3 g((c.NF + kFlushF - 1) / kFlushF, (c.netot + kFlushE - 1) / kFlushE);
    k_flux_flush<<<g, 256, 0, c.stream>>>(c.d_fring, c.d_cring, c.d_fl_poti, c.d_etot, c.netot, c.NF, chunk,
                                          c.fl_q, c.it, nullptr, 1, c.d_zcr, c.d_zcdr);
    LAUNCH_CHECK(c);
    // every pending iteration is in the accumulators now: clear the C slots so no
    // later slice flush adds them again
    cudaMemsetAsync(c.d_cring, 0, sizeof(float) * kFluxSlots * c.netot * 2, c.stream);
}

void launch_addv(Ctx &c, const double *psi, int g0, int g1)
{
    if (g1 <= g0) return;
    if (c.h32)
        k_addv<float><<<dim3((g1 - g0) * c.na, c.nchunk), 256, 0, c.stream>>>(devgrid(c), psi, c.d_h32, c.d_h,
                                                                               c.d_vsrc, g0 * c.na);
    else
        k_addv<double><<<dim3((g1 - g0) * c.na, c.nchunk), 256, 0, c.stream>>>(devgrid(c), psi, c.d_h, c.d_h,
                                                                                c.d_vsrc, g0 * c.na);
    LAUNCH_CHECK(c);
}

// the iteration and norm-slot base of a graph replay
// check's autocorrelation (main_madwave3.f:444-455) for iphoto >= 1:
// <psi0|psi_k> over a wave's points, block partial sums in a fixed order, then
// one block sums the partials in order (deterministic, as the norm trace)
constexpr int kAutoPer = 8;          // points per thread
__global__ void __launch_bounds__(256) k_auto_part(const double *__restrict__ psi0, const double *__restrict__ pk,
                                                   int64_t n, double *__restrict__ part)
{
    __shared__ double red[8];
    const int64_t i0 = (int64_t)blockIdx.x * 256 * kAutoPer + threadIdx.x;
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kAutoPer; k++) {
        const int64_t i = i0 + 256 * k;
        if (i < n) s = fma(psi0[i], pk[i], s);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int wv = 0; wv < 8; wv++) t += red[wv];
        part[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(256) k_auto_reduce(const double *__restrict__ part, int nb, double *const *norms_out,
                                                     const int64_t *__restrict__ cap, int w, int64_t slot,
                                                     const int64_t *__restrict__ base)
{
    if (base) slot += base[1];
    __shared__ double red[256];
    double s = 0.0;
    for (int i = threadIdx.x; i < nb; i += 256) s += part[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int k = 128; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0 && slot >= 0 && slot < cap[w]) norms_out[w][cap[w] + slot] = red[0];
}

void launch_autocorr(Ctx &c, int64_t slot)
{
    const int64_t sarg = c.capturing ? slot - c.cap_slot0 : slot;
    const int64_t *bp = c.capturing ? c.d_itbase : nullptr;
    for (size_t w = 0; w < c.waves.size(); w++) {
        const WaveTables &t = c.waves[w];
        if (t.iphoto < 1 || !c.wdev[w].psi0) continue;
        const int nb = (int)((t.ntot + 256 * kAutoPer - 1) / (256 * kAutoPer));
        k_auto_part<<<nb, 256, 0, c.stream>>>(c.wdev[w].psi0, c.d_pk + t.flat0, t.ntot, c.d_autopart);
        LAUNCH_CHECK(c);
        k_auto_reduce<<<1, 256, 0, c.stream>>>(c.d_autopart, nb, c.d_norm_ptrs, c.d_norm_cap, (int)w, sarg, bp);
        LAUNCH_CHECK(c);
    }
}

// Cvj / Cvjprod of one iteration into its slot of the history ring (FP64 source,
// or the mixed path's FP32 Cvj ring slot); graph replays add the block's first
// slot from base[1] as k_norms does
__global__ void k_cvj_keep(const double *__restrict__ src64, const float *__restrict__ src32, int n,
                           double *__restrict__ dst, int64_t cap, int64_t slot, const int64_t *__restrict__ base)
{
    if (base) slot += base[1];
    const int64_t s = slot % cap;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        dst[s * n + i] = src64 ? src64[i] : (double)src32[i];
}

void launch_cvj_keep(Ctx &c, int64_t it, int64_t slot)
{
    if (c.hist_cap <= 0) return;
    const int64_t sarg = c.capturing ? slot - c.cap_slot0 : slot;
    const int64_t *bp = c.capturing ? c.d_itbase : nullptr;
    if (c.d_cvjh && c.n2 > 1) {
        const int R = c.G * c.nj * c.nv;
        const float *s32 = c.d_cvring ? c.d_cvring + (size_t)(it % kFluxRing) * R : nullptr;
        k_cvj_keep<<<(R + 255) / 256, 256, 0, c.stream>>>(c.d_cvring ? nullptr : c.d_cvj, s32, R, c.d_cvjh,
                                                           c.hist_cap, sarg, bp);
        LAUNCH_CHECK(c);
    }
    for (size_t w = 0; w < c.wdev.size(); w++) {
        const ProdDev &d = c.wdev[w].prod;
        if (!d.cvjph || !d.cvjprod) continue;
        k_cvj_keep<<<(d.nrow + 255) / 256, 256, 0, c.stream>>>(d.cvjprod, nullptr, d.nrow, d.cvjph, c.hist_cap, sarg,
                                                               bp);
        LAUNCH_CHECK(c);
    }
}

__global__ void k_set_itbase(int64_t *base, int64_t it, int64_t slot)
{
    base[0] = it;
    base[1] = slot;
}

void launch_set_itbase(Ctx &c)
{
    k_set_itbase<<<1, 1, 0, c.stream>>>(c.d_itbase, c.it, c.norm_slot);
    LAUNCH_CHECK(c);
}

void launch_norms(Ctx &c, int64_t slot)
{
    k_norms<<<(int)c.waves.size(), 256, 0, c.stream>>>(c.d_normpart, c.d_wseg0, c.d_wseg1, c.nchunk,
                                                       c.d_norm_ptrs, c.d_norm_cap,
                                                       c.capturing ? slot - c.cap_slot0 : slot,
                                                       c.capturing ? c.d_itbase : nullptr);
    LAUNCH_CHECK(c);
}

void launch_totalflux(Ctx &c, int w, double *d_out, double *d_outelec)
{
    WaveTables &t = c.waves[w];
    WaveDev &wd = c.wdev[w];
    double ah1 = (c.grid.rfin1 - c.grid.rmis1) / (double)(c.n1 - 1);
    k_totalflux<<<(t.netot + 127) / 128, 128, 0, c.stream>>>(wd.zcr, wd.zcdr, wd.fl_block, wd.nelebas, t.nflux,
                                                             t.netot, c.ne, wd.reacfct, ah1, d_out, d_outelec);
    LAUNCH_CHECK(c);
}

// a deterministic bounded pattern (|p| <= 5e-4) for timing runs that need no physics
__global__ void k_fill_pattern(double *__restrict__ p, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint32_t h = (uint32_t)i * 2654435761u;
        h ^= h >> 15;
        p[i] = 1e-3 * ((double)(h & 0xFFFFu) / 65536.0 - 0.5);
    }
}

void launch_fill_pattern(Ctx &c, double *p, int64_t n)
{
    k_fill_pattern<<<1024, 256, 0, c.stream>>>(p, n);
    LAUNCH_CHECK(c);
}

// ---------------------------------------------------------------------------
// H psi without allocation (mw3_hphi_noalloc): the same kernels as launch_hphi,
// with the two scratch rectangles taken from one static device array.
// ---------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_noalloc_scratch[MW3_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
// device address of g_noalloc_scratch per device ordinal, looked up once with
// that device current; it stays valid while the device's primary context lives
static void *s_noalloc_ptr[kMaxDevices];
static std::mutex s_noalloc_mu;

template <typename T>
static void noalloc_hphi(Ctx &c, const WaveTables &t, unsigned char *scratch, const double *psi, double *hpsi)
{
    int na = c.na, n1 = c.n1, n2 = c.n2;
    int g0 = t.g0, g1 = t.g0 + t.ncan, ng = t.ncan;
    size_t rect = (size_t)n1 * n2;
    // kernels index rectangles and vectors by context-wide block and flat
    // offsets: shift the bases so the wave's first entry lands at the buffer start
    T *X = reinterpret_cast<T *>(scratch) - (size_t)g0 * na * rect;
    T *Y = reinterpret_cast<T *>(scratch) + (size_t)ng * na * rect - (size_t)g0 * na * rect;
    const double *P = psi - t.flat0;
    double *H = hpsi - t.flat0;
    DevGrid d = devgrid(c);
    d.xt = 0;                                  // the scratch rectangle keeps [r1][R]
    k_scatter<T><<<dim3(ng * na, c.nchunk), 256, 0, c.stream>>>(d, X, P, nullptr, g0 * na, nullptr);
    LAUNCH_CHECK(c);
    constexpr int BM = RowCfg<T>::BM, BN = RowCfg<T>::BN;
    int64_t row0 = (int64_t)g0 * na * n1, nrows = (int64_t)ng * na * n1;
    dim3 gr((unsigned)((nrows + BM - 1) / BM), ((n2 + 1) / 2 + BN - 1) / BN);
    const bool rader = sizeof(T) == 8 && c.d_rd_tw;
    if (rader)
        k_dst_rows_rader<false><<<rd_grid(), 256, 0, c.stream>>>(d, (const double *)X, (double *)Y, nullptr,
                                                                 rd_tab(c), g0 * na, ng * na);
    else
        k_dst_rows<T, false><<<gr, 256, 0, c.stream>>>(d, X, (const T *)c.d_S2, Y, nullptr, c.d_nopr1, row0, nrows);
    LAUNCH_CHECK(c);
    dim3 gc(ng * na, (n2 + COL_W - 1) / COL_W);
    k_dst_cols<T><<<gc, 256, col_smem(c, sizeof(T)), c.stream>>>(d, Y, (const T *)c.d_S1, c.d_S1off, c.d_nopr1,
                                                                  c.d_p2r1, c.d_p2r2, c.grid.radcutmax, g0 * na);
    LAUNCH_CHECK(c);
    if (rader)
        k_dst_rows_rader<true><<<rd_grid(), 256, 0, c.stream>>>(d, (const double *)Y, nullptr, H, rd_tab(c), g0 * na,
                                                                ng * na);
    else
        k_dst_rows<T, true><<<gr, 256, 0, c.stream>>>(d, Y, (const T *)c.d_S2, nullptr, H, c.d_nopr1, row0, nrows);
    LAUNCH_CHECK(c);
    k_quirk<double><<<ng * na, 128, 0, c.stream>>>(d, P, H, c.d_quirk_ptr, c.d_quirk, g0 * na);
    LAUNCH_CHECK(c);
    if (sizeof(T) == 4 && c.use_tc_ang) {
        launch_tc_ang(c, (const float *)X, H, g0, g1, false);   // its own scratch, [r1][R]
    } else if (na > 1) {
        dim3 gj(c.ncj, n1, ng);
        k_ang_j<T><<<gj, 256, angj_smem(c, sizeof(T)), c.stream>>>(d, X, (const T *)c.d_xj2, H, c.d_tj_ptr, c.d_tj,
                                                                    c.ncj, g0, c.ang_cw);
        LAUNCH_CHECK(c);
        dim3 gl(c.ncl, n2, ng);
        k_ang_l<T><<<gl, 256, angl_smem(c, sizeof(T)), c.stream>>>(d, X, (const T *)c.d_xl2p, H, c.d_tl_ptr, c.d_tl,
                                                                    c.d_cpl, c.ncl, g0, c.ang_cw);
        LAUNCH_CHECK(c);
    }
    launch_ecor<T, double>(c, d, (const T *)X, H, g0, g1);
    k_addv<double><<<dim3(ng * na, c.nchunk), 256, 0, c.stream>>>(d, P, H, H, c.d_vsrc, g0 * na);
    LAUNCH_CHECK(c);
    (void)g1;
}

}  // namespace mw3

extern "C" int mw3_hphi_noalloc(mw3_ctx *h, int32_t wave_id, const double *psi, double *hpsi)
{
    using namespace mw3;
    if (!h || !psi || !hpsi) return MW3_ERR_ARG;
    Ctx &c = h->c;
    if (wave_id < 0 || wave_id >= (int)c.waves.size()) {
        c.err = "mw3_hphi_noalloc: no such wave";
        return MW3_ERR_ARG;
    }
    if (!c.built) {
        c.err = "mw3_hphi_noalloc: device tables not built yet (call mw3_hphi, mw3_start or mw3_upload_state once)";
        return MW3_ERR_STATE;
    }
    const WaveTables &t = c.waves[wave_id];
    size_t tsz = c.fp64 ? sizeof(double) : sizeof(float);
    size_t rect_bytes = (size_t)t.ncan * c.na * c.n1 * c.n2 * tsz;
    if (rect_bytes > MW3_NOALLOC_SCRATCH_BYTES / 2) {
        c.err = "mw3_hphi_noalloc: the wave needs " + std::to_string(2 * rect_bytes) +
                " bytes of scratch, more than the static array's " + std::to_string((size_t)MW3_NOALLOC_SCRATCH_BYTES);
        return MW3_ERR_UNSUPPORTED;
    }
    // psi is read after hpsi is first written (the V psi term of the other
    // same-Omega blocks, the ir1 > nopr1 points), so the two must not overlap
    const char *pb = reinterpret_cast<const char *>(psi), *hb = reinterpret_cast<const char *>(hpsi);
    size_t vbytes = sizeof(double) * (size_t)t.ntot;
    if (pb < hb + vbytes && hb < pb + vbytes) {
        c.err = "mw3_hphi_noalloc: psi and hpsi overlap";
        return MW3_ERR_ARG;
    }
    int dev = 0;
    MW3_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        c.err = "mw3_hphi_noalloc: device index out of range";
        return MW3_ERR_UNSUPPORTED;
    }
    void *base = nullptr;
    {
        std::lock_guard<std::mutex> lock(s_noalloc_mu);
        if (!s_noalloc_ptr[dev]) {
            // once per device, with that device current: the device address of the array
            void *p = nullptr;
            MW3_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
            s_noalloc_ptr[dev] = p;
        }
        base = s_noalloc_ptr[dev];
    }
    unsigned char *scratch = static_cast<unsigned char *>(base);
    // the array keeps the previous call's contents; the psi rectangle must be
    // zero outside the stored points
    MW3_CUDA_TRY(cudaMemsetAsync(scratch, 0, rect_bytes, c.stream));
    if (c.fp64)
        noalloc_hphi<double>(c, t, scratch, psi, hpsi);
    else
        noalloc_hphi<float>(c, t, scratch, psi, hpsi);
    int rc = api_check_launch(c, "mw3_hphi_noalloc");
    if (rc) return rc;
    MW3_CUDA_TRY(cudaStreamSynchronize(c.stream));
    return api_check_device_flags(c, "mw3_hphi_noalloc");
}

namespace mw3 {

template void launch_scatter<double>(Ctx &, const double *, float *, int, int);
template void launch_scatter<float>(Ctx &, const double *, float *, int, int);
template void launch_hphi<double>(Ctx &, const double *, int, int);
template void launch_hphi<float>(Ctx &, const double *, int, int);
template void launch_update<double>(Ctx &, int);
template void launch_update<float>(Ctx &, int);
template void launch_build_kinetic<double>(Ctx &);
template void launch_build_kinetic<float>(Ctx &);

}  // namespace mw3
