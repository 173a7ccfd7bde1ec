// Radial kinetic term of the mixed path (difs T-part, SRC/mod_Hphi_01y2.f:752-832)
// as ONE kernel per (block, angle) slab, everything between reading psi and
// writing H kept on chip (tensor memory holds the intermediate products, R up
// to 256 points as two 128-lane tiles).
//
// With Xs = psi on the slab [r1 < nopr1][R], the reference computes (RODFT00
// along R, along r1, k-space scaling, back along r1 and R)
//   H = S1 ((S1 Xs S2) o F) S2 ,   F[r1][R] = min(p2r1 + p2r2, radcut) / (4 (nopr1+1)(npun2+1)).
// Four 128 x 128 tensor-core GEMMs, oriented so that each result can be read
// out of tensor memory row by row (a thread owns one lane) and written back as
// the next GEMM's K-major operand without a transpose:
//   D1[R][r1] = S2 Xs^T            A = S2 (bulk copy)      B = Xs rows (tensor copy) [R folded]
//   D2[R][r1] = D1 S1^T            A = D1 (tensor memory)  B = S1 (bulk copy)
//   D3[r1][R] = S1 (D2 o F^T)^T    A = S1 (bulk copy)      B = D2 o F^T (tensor memory)
//   D4[r1][R] = D3 S2              A = D3 (tensor memory)  B = S2 (bulk copy)        [R folded]
// so H[r1][R] = D4, written with lanes along r1 (stored points are r1-major runs).
// K streams in chunks of 16 through four shared-memory stages; the DST matrices
// are split on the host into TF32 hi/lo planes in the canonical K-major chunk
// layout and arrive by one bulk (TMA) copy per chunk.  3xTF32 products with
// FP32 accumulation as the other tensor-core kernels of the mixed path.
#include "mw3_internal.h"
#include "mw3_tc.cuh"

#include <cuda.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>

namespace mw3 {
namespace tc {

// The two products along R use the symmetry of DST-I,
//   S[n-1-i][k] = (-1)^k S[i][k]:
// with E_i = sum_{k even} S[i][k] x_k and O_i = sum_{k odd} S[i][k] x_k for
// i < h = ceil(n/2), y_i = E_i + O_i and y_{n-1-i} = E_i - O_i, so each is a
// pair of 128 x 128 products over the even and the odd half of K instead of a
// 256 x 256 one.  The products along r1 take N = nopr1 rounded up to 16.
//
// Pipeline: the four products form one sequence of K chunks of 16 per slab,
// streamed through four shared-memory stages by three warp roles (below).
// Every tcgen05.ld is executed by whole warps (its conditions depend on the
// warp only); lane-dependent choices are made on the loaded values.
constexpr int D2_KC = 16;
constexpr int D2_NS = 4;                                // stages
constexpr uint32_t D2_SBO = (D2_KC / 4) * 128;          // 512 B between 8-row groups
constexpr uint32_t D2_SMALL = 2 * 128 * D2_KC * 4;      // 16 KB: hi + lo, 128 rows x 16 k
constexpr uint32_t D2_SMALL_LO = D2_SMALL / 2;          // lo plane of a 128-row operand
constexpr uint32_t D2_BIGMAX = 2 * 256 * D2_KC * 4;     // 32 KB: hi + lo, 256 rows x 16 k
constexpr uint32_t D2_STAGE = D2_BIGMAX + D2_SMALL;     // 48 KB
constexpr uint32_t D2_BYTES = D2_NS * D2_STAGE;         // 192 KB
constexpr int D2_NKH = 128 / D2_KC;                     // K chunks of a 128-wide operand
constexpr size_t D2_CHUNK = D2_SMALL / 4;               // floats of one 128-row chunk (hi + lo)

struct Dst2Args {
    const float *X;               // rectangle [G][na][n1][n2]
    float *H;                     // H psi without V, FP32
    const float *s2fold;          // [parity][D2_NKH][hi, lo]: S2[i][2j+parity], i < 128, j chunk of 16
    const float *s1planes;        // S1 of each length, D2_NKH chunks of 16 columns
    const int64_t *s1off;         // [W][na]
    const int *nopr1;             // [W][na]
    const float *p2r1f, *p2r2f;   // [W][na][n1], [W][na][n2]
    float radcut;
    const int *mapT;              // [na][n2][n1]
    const int2 *rows;             // [na][n2][4]: stored-r1 bits of word w, index of its first stored point
    const int *rows_ok;           // [na]: every R row's indices run consecutively in r1
    int wave;                     // CTAs resident at once (one per SM): the next wave's slab is seg + wave
    const int64_t *foff;
    const int *blk_wave;
    int na, n1, n2, seg0;
    int *err;
};

// H at the stored points of one slab from D4 (E in tensor-memory columns 256 + i,
// O in 384 + i of lane m = r1 = 32 q + l): R = i takes E + O and R = n2-1-i takes
// E - O, for the 32 i of warp group sub.  When the angle's rows store their points
// consecutively in r1 order, a point's index is the row's count before word q plus
// the stored bits below l: srow, the angle's (bits, count) table staged in shared
// memory (8 KB), gives both in one broadcast read per row.  Otherwise (srow null)
// through the [R][r1] map: a coalesced 128-byte line per R, 128 KB per slab,
// prefetched into L1 while the last products run.
__device__ __forceinline__ void d2_prefetch_map(const Dst2Args &p, int a, int m, int nn, int h, int sub)
{
    const int n1 = p.n1, n2 = p.n2;
    const int *mT = p.mapT + (size_t)a * n2 * n1;
    if (m < nn) {
#pragma unroll 4
        for (int uu = 0; uu < 32; uu++) {
            int i = 32 * sub + uu;
            if (i < h) asm volatile("prefetch.global.L1 [%0];" ::"l"(mT + (size_t)i * n1 + m));
            if (i < n2 - h) asm volatile("prefetch.global.L1 [%0];" ::"l"(mT + (size_t)(n2 - 1 - i) * n1 + m));
        }
    }
}

// the angle's row table into shared memory (fill warps; visible after their next barrier)
__device__ __forceinline__ void d2_stage_rows(const Dst2Args &p, int a, int2 *srow, int nthreads)
{
    const int4 *src = reinterpret_cast<const int4 *>(p.rows + (size_t)a * p.n2 * 4);
    int4 *dst = reinterpret_cast<int4 *>(srow);
    for (int e = threadIdx.x; e < 2 * p.n2; e += nthreads) dst[e] = __ldg(src + e);
}

__device__ __forceinline__ void d2_store_h(const Dst2Args &p, int a, int64_t fo, int m, int nn, int h, int sub,
                                           uint32_t lrow, float hinv, const int2 *srow)
{
    const int n1 = p.n1, n2 = p.n2;
    const int q = m >> 5;
    const unsigned below = (1u << (m & 31)) - 1u, me = 1u << (m & 31);
    const int *mT = p.mapT + (size_t)a * n2 * n1;
#pragma unroll 1
    for (int cc = 0; cc < 4; cc++) {
        const int i0 = 32 * sub + 8 * cc;
        float e[8], o[8];
        tmem_ld8(lrow + 256u + (uint32_t)i0, e);
        tmem_ld8(lrow + 384u + (uint32_t)i0, o);
        if (srow) {
            if (m < nn) {
#pragma unroll
                for (int uu = 0; uu < 8; uu++) {
                    const int i = i0 + uu;
                    if (i < h) {
                        const int2 r = srow[i * 4 + q];
                        if (r.x & me) p.H[fo + r.y + __popc(r.x & below)] = (e[uu] + o[uu]) * hinv;
                    }
                    if (i < n2 - h) {
                        const int2 r = srow[(n2 - 1 - i) * 4 + q];
                        if (r.x & me) p.H[fo + r.y + __popc(r.x & below)] = (e[uu] - o[uu]) * hinv;
                    }
                }
            }
        } else {
            int is[8], id[8];
#pragma unroll
            for (int uu = 0; uu < 8; uu++) {
                const int i = i0 + uu;
                is[uu] = (m < nn && i < h) ? __ldg(mT + (size_t)i * n1 + m) : -1;
                id[uu] = (m < nn && i < n2 - h) ? __ldg(mT + (size_t)(n2 - 1 - i) * n1 + m) : -1;
            }
#pragma unroll
            for (int uu = 0; uu < 8; uu++) {
                if (is[uu] >= 0) p.H[fo + is[uu]] = (e[uu] + o[uu]) * hinv;
                if (id[uu] >= 0) p.H[fo + id[uu]] = (e[uu] - o[uu]) * hinv;
            }
        }
    }
}

// four values of one row into the hi plane at off and the lo plane lo_off further
__device__ __forceinline__ void d2_split4(unsigned char *hi, uint32_t lo_off, uint32_t off, float a, float b,
                                          float c, float d)
{
    float4 h = make_float4(tf32_hi(a), tf32_hi(b), tf32_hi(c), tf32_hi(d));
    float4 l = make_float4(a - h.x, b - h.y, c - h.z, d - h.w);
    *reinterpret_cast<float4 *>(hi + off) = h;
    *reinterpret_cast<float4 *>(hi + lo_off + off) = l;
}

// X rows r < nn, columns 2j + parity for j in [16 jc, 16 jc + 16), from the
// chunk's X tile (128 rows x 32 columns, one 128-byte row each, placed by the
// tensor copy with the 128-byte swizzle: 16-byte piece q of row r sits at piece
// q ^ (r & 7)).  Each of the 512 fill threads takes one (row, 4 j) group: the
// pieces 2 kg and 2 kg + 1 of its row hold both parities.  A quarter warp reads
// 8 consecutive rows, whose pieces the swizzle spreads over all banks, and
// writes one core matrix of the K-major operand.
__device__ __forceinline__ void d2_x_fill(const unsigned char *xt, unsigned char *dst, int parity, int nn)
{
    const int e = threadIdx.x, rest = e >> 3, kg = rest & 3, r = (rest >> 2) * 8 + (e & 7);
    const unsigned char *row = xt + r * 128;
    float4 a = *reinterpret_cast<const float4 *>(row + (((2 * kg) ^ (r & 7)) << 4));
    float4 b = *reinterpret_cast<const float4 *>(row + (((2 * kg + 1) ^ (r & 7)) << 4));
    if (r >= nn) a = b = make_float4(0.f, 0.f, 0.f, 0.f);
    if (parity == 0)
        d2_split4(dst, D2_SMALL_LO, kmaj_off(r, kg * 4, D2_KC), a.x, a.z, b.x, b.z);
    else
        d2_split4(dst, D2_SMALL_LO, kmaj_off(r, kg * 4, D2_KC), a.y, a.w, b.y, b.w);
}

// 2-D tensor copy of a box at (x, y) of the map into shared memory
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *mbar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        :
        : "r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(mbar))
        : "memory");
}

// L2 prefetch of one 2-D tile (no shared memory, no completion): the first
// product's X tiles start streaming from DRAM while the slab sets up
__device__ __forceinline__ void tma_prefetch_2d(const CUtensorMap *map, int x, int y)
{
    asm volatile("cp.async.bulk.prefetch.tensor.2d.L2.global.tile [%0, {%1, %2}];"
                 :
                 : "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y)
                 : "memory");
}

// Tensor memory (512 columns):
//   D1 = S2 Xs^T folded: E at [0,128), O at [128,256)   (lane i < h, column r1)
//   D2 = D1 S1^T:        R tile t at [256 + 128 t)       (lane R, column r1)
//   D3 = S1 (D2 o F^T)^T at [0, 256)                     (lane r1, column R)
//   D4 = D3 S2 folded:   E at [256,384), O at [384,512)  (lane r1, column i < h)
//
// Warp roles (576 threads): warps 0-15 build the register-side operand of each
// chunk (four warps per 32-lane quarter of tensor memory, each a quarter of
// the chunk) and write H; warp 16 issues the MMAs; warp 17 issues the bulk
// copies of the DST-matrix operands.  They meet only at two mbarriers per
// stage: full (the 16 fill-warp arrivals, the copy warp's arrival and the
// copied bytes) and empty (the MMAs that read the stage completed).  The MMA
// warp thus makes one shared-memory wait per chunk: while the tensor cores
// read their operands, every other shared-memory access of that warp takes a
// few hundred cycles (measured with clock stamps per chunk), and those waits,
// not the copies or the fills, set the chunk rate.
// Chunk t uses stage t % NS for the (t / NS)-th time, so every wait names the
// phase parity (t / NS) & 1; no role can run a full phase ahead of a waiter.
// The three roles walk the same chunk sequence as nested loops (product, then
// parity and K chunk), with no integer division per chunk.  After any wait
// runs out of time the CTA's shared failure flag makes every later wait return
// at once, so a fault ends the kernel instead of hanging it.
constexpr int D2_FILL = 16;                        // fill warps
constexpr int D2_WARPS = D2_FILL + 2;
constexpr int D2_MMA_WARP = D2_FILL, D2_COPY_WARP = D2_FILL + 1;

__device__ __forceinline__ void mbar_arrive1(uint64_t *mbar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" : : "r"(smem_u32(mbar)) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t a, uint32_t parity)
{
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.b32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    return done != 0;
}

// wait for a phase: the first test is the only shared-memory access on the fast
// path; the failure flag and the clock are read on the slow path only (every
// 32nd test), so a failure elsewhere in the CTA still ends this wait quickly
__device__ __forceinline__ bool d2_wait(uint64_t *mbar, uint32_t parity, volatile int *fail)
{
    const uint32_t a = smem_u32(mbar);
    if (mbar_try(a, parity)) return true;
    const long long t0 = clock64();
    for (int it = 1;; it++) {
        if (mbar_try(a, parity)) return true;
        if ((it & 31) == 0) {
            if (*fail) return false;
            if (clock64() - t0 > kWaitCycles) {
                *fail = 1;
                return false;
            }
        }
    }
}

// the chunk sequence of one slab: product gi in 0..3, parity half par (products
// along R) and K chunk jc; f(t, gi, par, jc) is called for t = 0, 1, ...  The
// first product alternates the parities per K chunk, so both of its chunks use
// one load of X; E and O are separate accumulators, so the order is free.
template <typename F>
__device__ __forceinline__ void d2_for_chunks(int nkh, int nkr, F &&f)
{
    int t = 0;
    for (int jc = 0; jc < nkh; jc++)
        for (int par = 0; par < 2; par++) f(t++, 0, par, jc);
    for (int jc = 0; jc < nkr; jc++) f(t++, 1, 0, jc);
    for (int jc = 0; jc < nkr; jc++) f(t++, 2, 0, jc);
    for (int par = 0; par < 2; par++)
        for (int jc = 0; jc < nkh; jc++) f(t++, 3, par, jc);
}

__global__ void __launch_bounds__(D2_WARPS * 32, 1) k_tc_dst2d(Dst2Args p, const __grid_constant__ CUtensorMap xmap)
{
    extern __shared__ __align__(1024) unsigned char smraw[];
    unsigned char *sm = smraw + ((1024 - (smem_u32(smraw) & 1023)) & 1023);
    uint64_t *full = reinterpret_cast<uint64_t *>(sm + D2_BYTES);
    uint64_t *empty = full + D2_NS;
    uint64_t *xfull = empty + D2_NS;                    // the X tile of a first-product chunk landed
    uint32_t *slot = reinterpret_cast<uint32_t *>(xfull + D2_NS);
    float *s_p1f = reinterpret_cast<float *>(sm + D2_BYTES + 128);   // the slab's r1 momenta
    int2 *s_rows = reinterpret_cast<int2 *>(sm + D2_BYTES + 1024);   // the angle's row table [n2][4]
    volatile int *fail = reinterpret_cast<volatile int *>(slot + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int na = p.na, n1 = p.n1, n2 = p.n2;
    const int h = (n2 + 1) >> 1;                        // rows i < h: E + O; row n2-1-i: E - O
    const int nkh = (h + D2_KC - 1) / D2_KC;            // K chunks of one parity half
    const int seg = p.seg0 + blockIdx.x;
    if (warp == D2_COPY_WARP && lane == 0)
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&xmap)) : "memory");
    if (warp == 0) tmem_alloc(slot, 512);
    if (threadIdx.x == 0) {
        for (int i = 0; i < D2_NS; i++) {
            mbar_init(&full[i], D2_FILL + 1);
            mbar_init(&empty[i], 1);
            mbar_init(&xfull[i], 1);
        }
        *fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tb = *slot;
    const int NT = (n2 + 127) / 128;                    // R tiles of D2 and of the D3 columns
    const int RB = 128 * NT;
    const uint32_t big_lo = (uint32_t)RB * D2_KC * 4;   // lo plane of an RB-row operand
    const int g = seg / na, a = seg % na, w = p.blk_wave[g];
    const int nn = p.nopr1[w * na + a];
    const int nnp = (nn + 15) & ~15;                    // N of the products along r1
    const int nkr = (nn + D2_KC - 1) / D2_KC;           // K chunks of the products along r1
    const int total = 4 * nkh + 2 * nkr;
    const float *S1p = p.s1planes + p.s1off[w * na + a];
    int copies = 0;                                     // copies issued (copy warp, lane 0)

    if (warp == D2_COPY_WARP) {
        // ---- bulk copies of the DST-matrix operands ----
        if (lane == 0)
            d2_for_chunks(nkh, nkr, [&](int t, int gi, int par, int jc) {
                if (*fail) return;
                const int s = t & (D2_NS - 1), u = t >> 2;
                if (t >= D2_NS && !d2_wait(&empty[s], (u - 1) & 1, fail)) return;
                unsigned char *big = sm + s * D2_STAGE, *small = big + D2_BIGMAX;
                const bool alongR = (gi == 0 || gi == 3);
                const float *src = alongR ? p.s2fold + (size_t)(par * D2_NKH + jc) * D2_CHUNK
                                          : S1p + (size_t)jc * D2_CHUNK;
                if (gi == 0) {
                    // the X tile of this chunk (rows of the slab, 32 columns) behind the S2 chunk
                    mbar_expect_tx(&xfull[s], D2_SMALL);
                    tma_load_2d(big + D2_SMALL, &xmap, 32 * jc, seg * n1, &xfull[s]);
                }
                mbar_expect_tx(&full[s], D2_SMALL);
                bulk_g2s(alongR ? big : small, src, D2_SMALL, &full[s]);
                copies = t + 1;
            });
    } else if (warp == D2_MMA_WARP) {
        // ---- MMA issue: descriptors built once, advanced by 16-byte units ----
        if (lane == 0) {
            const uint64_t k16 = 256 >> 4;                  // one K step of 8 (two core matrices)
            const uint64_t d0 = sdesc(smem_u32(sm), 128, D2_SBO);
            const uint64_t stage16 = D2_STAGE >> 4, small16 = D2_BIGMAX >> 4;
            const uint64_t lo128 = D2_SMALL_LO >> 4, loRB = big_lo >> 4, tile16 = (16 * D2_SBO) >> 4;
            const uint32_t id_nn = idesc_tf32(128, nnp), id_rb = idesc_tf32(128, RB), id_128 = idesc_tf32(128, 128);
            d2_for_chunks(nkh, nkr, [&](int t, int gi, int par, int jc) {
                const int s = t & (D2_NS - 1), u = t >> 2;
                const bool ok = d2_wait(&full[s], u & 1, fail);
                fence_after_sync();
                if (ok) {
                    const uint64_t bg = d0 + (uint64_t)s * stage16, sl = bg + small16;
#pragma unroll
                    for (int ks = 0; ks < D2_KC / 8; ks++) {
                        const uint64_t o = ks * k16;
                        const int acc0 = (jc > 0 || ks > 0) ? 1 : 0;
                        if (gi == 0) {
                            // E or O: M = 128 (i), N = nnp (r1): A = folded S2 (big), B = Xs (small)
                            const uint32_t d = tb + 128u * par;
                            mma_tf32(d, bg + o, sl + o, id_nn, acc0);
                            mma_tf32(d, bg + o, sl + lo128 + o, id_nn, 1);
                            mma_tf32(d, bg + lo128 + o, sl + o, id_nn, 1);
                        } else if (gi == 1) {
                            // per R tile: M = 128, N = nnp: A = D1 rows (big), B = S1 (small)
                            for (int tt = 0; tt < NT; tt++) {
                                const uint64_t at = bg + tt * tile16;
                                const uint32_t d = tb + 256u + 128u * tt;
                                mma_tf32(d, at + o, sl + o, id_nn, acc0);
                                mma_tf32(d, at + o, sl + lo128 + o, id_nn, 1);
                                mma_tf32(d, at + loRB + o, sl + o, id_nn, 1);
                            }
                        } else if (gi == 2) {
                            // M = 128 (r1), N = RB (R): A = S1 (small), B = scaled D2 rows (big)
                            mma_tf32(tb, sl + o, bg + o, id_rb, acc0);
                            mma_tf32(tb, sl + o, bg + loRB + o, id_rb, 1);
                            mma_tf32(tb, sl + lo128 + o, bg + o, id_rb, 1);
                        } else {
                            // E or O: M = 128 (r1), N = 128 (i): A = D3 columns (small), B = folded S2 (big)
                            const uint32_t d = tb + 256u + 128u * par;
                            mma_tf32(d, sl + o, bg + o, id_128, acc0);
                            mma_tf32(d, sl + o, bg + lo128 + o, id_128, 1);
                            mma_tf32(d, sl + lo128 + o, bg + o, id_128, 1);
                        }
                    }
                }
                mma_commit(&empty[s]);        // also after a failure, so no waiter is left behind
            });
        }
    } else {
        // ---- operand fills (warps 0-15) and the H epilogue ----
        // warp = 4 sub + q4: q4 the 32-lane quarter of tensor memory it reads, sub
        // the quarter of each chunk it builds
        const int q4 = warp & 3, sub = warp >> 2;
        const int m = q4 * 32 + lane;                   // the tensor-memory lane this thread reads
        const uint32_t lrow = tb + ((uint32_t)(q4 * 32) << 16);
        const float divi = 1.0f / (4.0f * (float)(nn + 1) * (float)(n2 + 1));
        {
            // the r1 momenta of the slab into shared memory (read 8 at a time by the third
            // product) and, when the angle has one, its row table (read by the H write)
            const float *p1f = p.p2r1f + ((size_t)w * na + a) * n1;
            if (threadIdx.x < 128) s_p1f[threadIdx.x] = threadIdx.x < nn ? p1f[threadIdx.x] : 0.f;
            if (p.rows_ok[a]) d2_stage_rows(p, a, s_rows, D2_FILL * 32);
            asm volatile("bar.sync 1, %0;" ::"n"(D2_FILL * 32) : "memory");
        }
        // second and third products: sub & 1 picks the row set, sub >> 1 the 8-column half
        const int rset = sub & 1, colh = sub >> 1;
        const int rR = 128 * rset + m;                  // the R row this thread fills in the third product
        const float e2 = (rset < NT && rR < n2) ? p.p2r2f[((size_t)w * na + a) * n2 + rR] : 0.f;
        const float radcut = p.radcut;
        // second product rows: rset 0 the sum rows R = i, rset 1 the difference rows R = n2-1-i
        const bool on2 = rset == 0 ? (m < h) : (m < n2 - h);
        const int R2 = rset == 0 ? m : n2 - 1 - m;
        const float sg2 = rset == 0 ? 1.f : -1.f;
        d2_for_chunks(nkh, nkr, [&](int t, int gi, int par, int jc) {
            const int s = t & (D2_NS - 1), u = t >> 2;
            unsigned char *big = sm + s * D2_STAGE, *small = big + D2_BIGMAX;
            if (jc == 0 && par == 0 && gi > 0) {
                // this product reads the previous one from tensor memory: its last chunk done
                d2_wait(&empty[(t - 1) & (D2_NS - 1)], ((t - 1) >> 2) & 1, fail);
                fence_after_sync();
            }
            if (t >= D2_NS) d2_wait(&empty[s], (u - 1) & 1, fail);   // the MMAs of chunk t - NS read this stage
            const int k0 = jc * D2_KC;
            if (gi == 0) {
                // B = Xs columns of this parity (rows r1) into the small slot, from the X
                // tile the copy warp placed behind the S2 chunk (the first product takes the
                // first uses of every stage, so u counts this barrier's phases too)
                d2_wait(&xfull[s], u & 1, fail);
                d2_x_fill(big + D2_SMALL, small, par, nn);
            } else if (gi == 1) {
                // A = D1 rows R into the big slot from 8 of the E and O columns of lane i
                // (all lanes load; lanes without a row store nothing)
                const int kc = k0 + 8 * colh;
                float e[8], o[8];
                tmem_ld8(lrow + (uint32_t)kc, e);
                tmem_ld8(lrow + 128u + (uint32_t)kc, o);
                if (on2) {
                    const bool full = kc + 8 <= nn;
#pragma unroll
                    for (int j = 0; j < 2; j++) {
                        float tv[4];
#pragma unroll
                        for (int uu = 0; uu < 4; uu++) {
                            float x = e[4 * j + uu] + sg2 * o[4 * j + uu];
                            tv[uu] = (full || kc + 4 * j + uu < nn) ? x : 0.f;
                        }
                        d2_split4(big, big_lo, kmaj_off(R2, 8 * colh + 4 * j, D2_KC), tv[0], tv[1], tv[2], tv[3]);
                    }
                }
            } else if (gi == 2) {
                // B = (D2 o F^T) rows R into the big slot: R tile rset, 8 columns (warp-uniform test)
                if (rset < NT) {
                    const int kc = k0 + 8 * colh;
                    float v[8];
                    tmem_ld8(lrow + 256u + 128u * rset + (uint32_t)kc, v);
                    float pv[8];
#pragma unroll
                    for (int j = 0; j < 2; j++) {
                        float4 q = *reinterpret_cast<const float4 *>(s_p1f + kc + 4 * j);
                        pv[4 * j] = q.x; pv[4 * j + 1] = q.y; pv[4 * j + 2] = q.z; pv[4 * j + 3] = q.w;
                    }
                    const bool full = kc + 8 <= nn && rR < n2;
#pragma unroll
                    for (int i = 0; i < 8; i++) {
                        float ek = fminf(pv[i] + e2, radcut);
                        float x = v[i] * ek * divi;
                        v[i] = (full || (kc + i < nn && rR < n2)) ? x : 0.f;
                    }
#pragma unroll
                    for (int j = 0; j < 2; j++)
                        d2_split4(big, big_lo, kmaj_off(rR, 8 * colh + 4 * j, D2_KC), v[4 * j], v[4 * j + 1],
                                  v[4 * j + 2], v[4 * j + 3]);
                }
            } else {
                // A = D3 columns 2j + parity (rows r1) into the small slot; warp sub reads the
                // 8 consecutive columns of j in [k0 + 4 sub, k0 + 4 sub + 4) and keeps 4
                float v[8];
                const int col0 = 2 * k0 + 8 * sub;
                tmem_ld8(lrow + (uint32_t)col0, v);
                const bool full = col0 + 8 <= n2;
                float tv[4];
#pragma unroll
                for (int uu = 0; uu < 4; uu++) {
                    const int cc = 2 * uu;                     // register index fixed at compile time
                    float x = par == 0 ? v[cc] : v[cc + 1];
                    tv[uu] = (full || col0 + cc + par < n2) ? x : 0.f;
                }
                d2_split4(small, D2_SMALL_LO, kmaj_off(m, 4 * sub, D2_KC), tv[0], tv[1], tv[2], tv[3]);
            }
            // make the generic shared-memory writes visible to the tensor cores, order the
            // tensor-memory loads before the arrival, then one arrival per warp
            fence_async_smem();
            fence_before_sync();
            __syncwarp();
            if (lane == 0) mbar_arrive1(&full[s]);
        });
        // ---- H at the stored points: lane r1; R = i takes E + O, R = n2-1-i takes E - O ----
        const int2 *srow = p.rows_ok[a] ? s_rows : nullptr;
        if (!srow) d2_prefetch_map(p, a, m, nn, h, sub);
        d2_wait(&empty[(total - 1) & (D2_NS - 1)], ((total - 1) >> 2) & 1, fail);
        fence_after_sync();
        if (!*fail) d2_store_h(p, a, p.foff[seg], m, nn, h, sub, lrow, 1.f, srow);
    }
    // before shared and tensor memory are released, the async work this CTA issued
    // must be done: the copy warp waits for its last copy, the MMA warp for its
    // last commit (which tracks all its MMAs); both phases were issued, so these
    // bounded waits end at once in a normal run and soon after a failure
    if (lane == 0 && warp == D2_COPY_WARP && copies > 0)
        mbar_wait(&full[(copies - 1) & (D2_NS - 1)], ((copies - 1) >> 2) & 1);
    if (lane == 0 && warp == D2_MMA_WARP) mbar_wait(&empty[(total - 1) & (D2_NS - 1)], ((total - 1) >> 2) & 1);
    fence_before_sync();
    __syncthreads();
    if (threadIdx.x == 0 && *fail) atomicExch(p.err, 1);
    if (warp == 0) tmem_dealloc(tb, 512);
}

// ===========================================================================
// The same chain as split-FP16 products (kind::f16, FP32 accumulation).
//
// FP16 and TF32 carry the same 10-bit mantissa, so x ~= hi + lo with hi, lo in
// FP16 keeps 22 bits like the TF32 split, and Ahi Bhi + Ahi Blo + Alo Bhi has the
// error of the 3xTF32 form; kind::f16 runs at twice the kind::tf32 rate.  FP16's
// exponent range is narrow, so every operand is scaled by a power of two that
// puts its largest element in [2^11, 2^12): the lo part of an element within
// 2^-11 of that maximum then stays a normal FP16 number, and the absolute error
// of any element is at most 2^-25 (half the spacing of the FP16 subnormals)
// against a maximum of 2^11, so the split keeps 22 bits of every element that
// matters to the product:
//   DST matrices    x 2^12 (entries 2 sin(.) are bounded by 2; host planes);
//   Xs              x 2^(12 - e), xmax < 2^e the slab's largest |X|, which the
//                   kernels that write X leave in xmax[slab] (atomicMax of the
//                   bits; this kernel reads it and clears it);
//   D1, D3          x 2^-20: |D1| <= 2^12 * 2^13 * 256 terms, and |D3| the same
//                   with the normalised D2 o F below; the largest element of
//                   either is at least that of one 2 sin(.) x 2^12 term times the
//                   largest operand element (2^25 -> 2^5), so an element within
//                   2^-8 of it keeps a normal lo part;
//   D2 o F          x 2^(12 - e) with e from the slab's largest |element|, which
//                   the fill warps read out of tensor memory when the second
//                   product completes and reduce across the CTA (F's bound,
//                   radcut / (4 (nn+1)(n2+1)), sits up to 2^10 above the F of a
//                   smooth packet's spectrum, and with D2's own slack a fixed
//                   scale left this operand up to 2^16 low, its lo parts in FP16
//                   subnormals: 1e-4 relative error in H psi);
// and H is D4 times the inverse of the product of the scales, again a power of
// two.  A K chunk is 32 FP16 values, the same 64 bytes per row as the 16 TF32
// values of the TF32 form, so operands and DST-matrix chunks keep their byte
// layout while a slab takes half as many chunks (and MMA-warp waits); with the
// X tile of a first-product chunk now 64 R columns (two 32-column tensor
// copies), a stage is 64 KB and three stages fill the same 192 KB.
constexpr int H_KC = 32;                                // FP16 values of K per chunk
constexpr int H_NS = 3;                                 // stages
constexpr uint32_t H_SBO = (H_KC / 8) * 128;            // 512 B between 8-row groups
constexpr uint32_t H_SMALL = 2 * 128 * H_KC * 2;        // 16 KB: hi + lo, 128 rows
constexpr uint32_t H_SMALL_LO = H_SMALL / 2;
constexpr uint32_t H_BIG = 2 * 256 * H_KC * 2;          // 32 KB: hi + lo, 256 rows
constexpr uint32_t H_XT = 16384;                        // one 128 x 32 FP32 X tile
constexpr uint32_t H_STAGE = 65536;                     // big [0, 32K), X tiles [16K, 48K), small [48K, 64K)
constexpr uint32_t H_SMALL_AT = 49152;
constexpr uint32_t H_BYTES = H_NS * H_STAGE;            // 192 KB
constexpr int H_NKH = 128 / H_KC;                       // K chunks of a 128-wide operand
constexpr size_t H_CHUNK = H_SMALL / 2;                 // halves of one 128-row chunk (hi + lo)
constexpr int H_S_EXP = 12;                             // the DST matrices' scale 2^12
static_assert(H_SMALL == D2_SMALL && H_SBO == D2_SBO, "FP16 chunks keep the TF32 chunks' bytes");

__device__ __forceinline__ uint32_t kmaj16_off(int r, int k)
{
    return (uint32_t)((r & 7) * 16 + (r >> 3) * H_SBO + (k & 7) * 2 + (k >> 3) * 128);
}

// eight consecutive k values of one row (already scaled) into the hi plane at
// off and the lo plane lo_off further: hi = fp16(x), lo = fp16(x - hi)
__device__ __forceinline__ uint32_t h2_bits(__half2 x) { return *reinterpret_cast<const uint32_t *>(&x); }

// hi and lo of two values, packed (two values per cvt, the lower k in the low half)
__device__ __forceinline__ void h_split2(float a, float b, uint32_t &h, uint32_t &l)
{
    const __half2 hh = __floats2half2_rn(a, b);
    const float2 hf = __half22float2(hh);
    h = h2_bits(hh);
    l = h2_bits(__floats2half2_rn(a - hf.x, b - hf.y));
}

// eight consecutive k values of one row (already scaled) into the hi plane at
// off and the lo plane lo_off further: hi = fp16(x), lo = fp16(x - hi)
__device__ __forceinline__ void h_split8(unsigned char *hi, uint32_t lo_off, uint32_t off, float v0, float v1,
                                         float v2, float v3, float v4, float v5, float v6, float v7)
{
    uint32_t h0, h1, h2, h3, l0, l1, l2, l3;
    h_split2(v0, v1, h0, l0);
    h_split2(v2, v3, h1, l1);
    h_split2(v4, v5, h2, l2);
    h_split2(v6, v7, h3, l3);
    *reinterpret_cast<uint4 *>(hi + off) = make_uint4(h0, h1, h2, h3);
    *reinterpret_cast<uint4 *>(hi + lo_off + off) = make_uint4(l0, l1, l2, l3);
}

#define H_SPLIT8(dst, lo, off, v, o) \
    h_split8(dst, lo, off, v[o], v[o + 1], v[o + 2], v[o + 3], v[o + 4], v[o + 5], v[o + 6], v[o + 7])

// instruction descriptor of kind::f16 with FP16 A and B, FP32 accumulate, K-major
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N)
{
    return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t dtmem, uint64_t ad, uint64_t bd, uint32_t idesc, int accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        :
        : "r"(dtmem), "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate));
}

// the chunk sequence as d2_for_chunks, with the stage s and its phase parity ph
// carried along (three stages: no power of two)
template <typename F>
__device__ __forceinline__ void h_for_chunks(int nkh, int nkr, F &&f)
{
    int t = 0, s = 0, ph = 0;
    auto step = [&](int gi, int par, int jc) {
        f(t, s, ph, gi, par, jc);
        t++;
        if (++s == H_NS) {
            s = 0;
            ph ^= 1;
        }
    };
    for (int jc = 0; jc < nkh; jc++)
        for (int par = 0; par < 2; par++) step(0, par, jc);
    for (int jc = 0; jc < nkr; jc++) step(1, 0, jc);
    for (int jc = 0; jc < nkr; jc++) step(2, 0, jc);
    for (int par = 0; par < 2; par++)
        for (int jc = 0; jc < nkh; jc++) step(3, par, jc);
}

struct Dst2hArgs {
    Dst2Args b;                   // the TF32 kernel's arguments (matrix planes unused)
    const __half *s2fold;         // [parity][H_NKH][hi, lo] x 2^12
    const __half *s1planes;       // S1 of each length, H_NKH chunks of 32 columns, x 2^12
    unsigned *xmax;               // [G na]: bits of the slab's largest |X|, cleared here
    int xt;                       // rectangle layout: 0 [..][r1][R], 1 [..][R][r1] (the tensor map's)
};

__global__ void __launch_bounds__(D2_WARPS * 32, 1) k_tc_dst2d_h(Dst2hArgs P, const __grid_constant__ CUtensorMap xmap)
{
    extern __shared__ __align__(1024) unsigned char smraw[];
    unsigned char *sm = smraw + ((1024 - (smem_u32(smraw) & 1023)) & 1023);
    uint64_t *full = reinterpret_cast<uint64_t *>(sm + H_BYTES);
    uint64_t *empty = full + H_NS;
    uint64_t *xfull = empty + H_NS;
    uint32_t *slot = reinterpret_cast<uint32_t *>(xfull + H_NS);
    float *s_p1f = reinterpret_cast<float *>(sm + H_BYTES + 128);
    unsigned *s_red = reinterpret_cast<unsigned *>(sm + H_BYTES + 640);    // largest |D2 o F|
    int2 *s_rows = reinterpret_cast<int2 *>(sm + H_BYTES + 1024);          // the angle's row table [n2][4]
    volatile int *fail = reinterpret_cast<volatile int *>(slot + 1);
    const Dst2Args &p = P.b;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int na = p.na, n1 = p.n1, n2 = p.n2;
    const int h = (n2 + 1) >> 1;
    const int nkh = (h + H_KC - 1) / H_KC;
    const int seg = p.seg0 + blockIdx.x;
    if (warp == D2_COPY_WARP && lane == 0)
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&xmap)) : "memory");
    if (warp == 0) tmem_alloc(slot, 512);
    if (threadIdx.x == 0) {
        for (int i = 0; i < H_NS; i++) {
            mbar_init(&full[i], D2_FILL + 1);
            mbar_init(&empty[i], 1);
            mbar_init(&xfull[i], 1);
        }
        *fail = 0;
        s_red[0] = s_red[1] = s_red[2] = s_red[3] = 0u;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tb = *slot;
    const int NT = (n2 + 127) / 128;
    const int RB = 128 * NT;
    const uint32_t big_lo = (uint32_t)RB * H_KC * 2;    // lo plane of an RB-row operand
    const int g = seg / na, a = seg % na, w = p.blk_wave[g];
    const int nn = p.nopr1[w * na + a];
    const int nnp = (nn + 15) & ~15;
    const int nkr = (nn + H_KC - 1) / H_KC;
    const int total = 4 * nkh + 2 * nkr;
    const __half *S1p = P.s1planes + p.s1off[w * na + a];
    int copies = 0;

    if (warp == D2_COPY_WARP) {
        // once this slab's X copies are issued, the X of the slab the next wave of CTAs
        // takes (one CTA per SM, issued in order) streams into L2, so that slab's first
        // product finds its tiles there instead of waiting on DRAM chunk by chunk
        const int nxt = (int)blockIdx.x + p.wave;
        if (lane == 0)
            h_for_chunks(nkh, nkr, [&](int t, int s, int ph, int gi, int par, int jc) {
                if (*fail) return;
                if (t >= H_NS && !d2_wait(&empty[s], ph ^ 1, fail)) return;
                unsigned char *st = sm + (size_t)s * H_STAGE;
                const bool alongR = (gi == 0 || gi == 3);
                const __half *src = alongR ? P.s2fold + (size_t)(par * H_NKH + jc) * H_CHUNK
                                           : S1p + (size_t)jc * H_CHUNK;
                if (gi == 0 && par == 0) {
                    // the 64 R of this K chunk (both parities) behind the par 0 S2 chunk: two
                    // 32-R x 128-r1 tiles, or with the transposed rectangle four 32-r1 x
                    // 64-R tiles; the fill splits both parities from them
                    mbar_expect_tx(&xfull[s], 2 * H_XT);
                    if (P.xt) {
#pragma unroll
                        for (int q = 0; q < 4; q++)
                            tma_load_2d(st + 16384 + q * 8192, &xmap, 32 * q, seg * n2 + 64 * jc, &xfull[s]);
                    } else {
                        tma_load_2d(st + 16384, &xmap, 64 * jc, seg * n1, &xfull[s]);
                        tma_load_2d(st + 32768, &xmap, 64 * jc + 32, seg * n1, &xfull[s]);
                    }
                }
                mbar_expect_tx(&full[s], H_SMALL);
                bulk_g2s(alongR ? st : st + H_SMALL_AT, src, H_SMALL, &full[s]);
                copies = t + 1;
                if (t == 2 * nkh - 1 && nxt < (int)gridDim.x) {
                    if (P.xt) {
                        for (int j = 0; j < nkh; j++)
                            for (int q = 0; q < 4; q++) tma_prefetch_2d(&xmap, 32 * q, (seg + p.wave) * n2 + 64 * j);
                    } else {
                        for (int j = 0; j < 2 * nkh; j++) tma_prefetch_2d(&xmap, 32 * j, (seg + p.wave) * n1);
                    }
                }
            });
    } else if (warp == D2_MMA_WARP) {
        if (lane == 0) {
            const uint64_t k16 = 256 >> 4;                  // one K step of 16 (two core matrices)
            const uint64_t d0 = sdesc(smem_u32(sm), 128, H_SBO);
            const uint64_t stage16 = H_STAGE >> 4, small16 = H_SMALL_AT >> 4;
            const uint64_t lo128 = H_SMALL_LO >> 4, loRB = big_lo >> 4, tile16 = (16 * H_SBO) >> 4;
            const uint32_t id_nn = idesc_f16(128, nnp), id_rb = idesc_f16(128, RB), id_128 = idesc_f16(128, 128);
            h_for_chunks(nkh, nkr, [&](int t, int s, int ph, int gi, int par, int jc) {
                const bool ok = d2_wait(&full[s], ph, fail);
                fence_after_sync();
                if (ok) {
                    const uint64_t bg = d0 + (uint64_t)s * stage16, sl = bg + small16;
#pragma unroll
                    for (int ks = 0; ks < H_KC / 16; ks++) {
                        const uint64_t o = ks * k16;
                        const int acc0 = (jc > 0 || ks > 0) ? 1 : 0;
                        if (gi == 0) {
                            const uint32_t d = tb + 128u * par;
                            mma_f16(d, bg + o, sl + o, id_nn, acc0);
                            mma_f16(d, bg + o, sl + lo128 + o, id_nn, 1);
                            mma_f16(d, bg + lo128 + o, sl + o, id_nn, 1);
                        } else if (gi == 1) {
                            for (int tt = 0; tt < NT; tt++) {
                                const uint64_t at = bg + tt * tile16;
                                const uint32_t d = tb + 256u + 128u * tt;
                                mma_f16(d, at + o, sl + o, id_nn, acc0);
                                mma_f16(d, at + o, sl + lo128 + o, id_nn, 1);
                                mma_f16(d, at + loRB + o, sl + o, id_nn, 1);
                            }
                        } else if (gi == 2) {
                            mma_f16(tb, sl + o, bg + o, id_rb, acc0);
                            mma_f16(tb, sl + o, bg + loRB + o, id_rb, 1);
                            mma_f16(tb, sl + lo128 + o, bg + o, id_rb, 1);
                        } else {
                            const uint32_t d = tb + 256u + 128u * par;
                            mma_f16(d, sl + o, bg + o, id_128, acc0);
                            mma_f16(d, sl + o, bg + lo128 + o, id_128, 1);
                            mma_f16(d, sl + lo128 + o, bg + o, id_128, 1);
                        }
                    }
                }
                mma_commit(&empty[s]);
            });
        }
    } else {
        const int q4 = warp & 3, sub = warp >> 2;
        const int m = q4 * 32 + lane;
        const uint32_t lrow = tb + ((uint32_t)(q4 * 32) << 16);
        const float divi = 1.0f / (4.0f * (float)(nn + 1) * (float)(n2 + 1));
        // the slab's scales (powers of two, see above)
        const float xm = __uint_as_float(P.xmax[seg]);
        int ex = 0;
        if (xm > 0.f) frexpf(xm, &ex);                  // xm < 2^ex
        const int sx_exp = min(100, max(-100, 12 - ex));
        const float sx = ldexpf(1.f, sx_exp);
        int s_exp = sx_exp - 40;                        // sum of the operand scales' exponents (D1, D3: -20)
        constexpr float a13 = 1.f / 1048576.f;          // 2^-20
        float sc2 = 1.f;                                // D2 o F's scale, set when the second product completes
        {
            const float *p1f = p.p2r1f + ((size_t)w * na + a) * n1;
            if (threadIdx.x < 128) s_p1f[threadIdx.x] = threadIdx.x < nn ? p1f[threadIdx.x] : 0.f;
            if (p.rows_ok[a]) d2_stage_rows(p, a, s_rows, D2_FILL * 32);
            asm volatile("bar.sync 1, %0;" ::"n"(D2_FILL * 32) : "memory");
        }
        const int rset = sub & 1, colq = sub >> 1;
        const int rR = 128 * rset + m;
        const float e2 = (rset < NT && rR < n2) ? p.p2r2f[((size_t)w * na + a) * n2 + rR] : 0.f;
        const float radcut = p.radcut;
        const bool on2 = rset == 0 ? (m < h) : (m < n2 - h);
        const int R2 = rset == 0 ? m : n2 - 1 - m;
        const float sg2 = rset == 0 ? 1.f : -1.f;
        int pt = -1, pph = 0;                           // the previous chunk's stage and parity
        h_for_chunks(nkh, nkr, [&](int t, int s, int ph, int gi, int par, int jc) {
            unsigned char *st = sm + (size_t)s * H_STAGE, *big = st, *small = st + H_SMALL_AT;
            if (jc == 0 && par == 0 && gi > 0) {
                d2_wait(&empty[pt], pph, fail);
                fence_after_sync();
                // the second product is complete: the largest |D2 o F| this thread will
                // write, over the chunks below (loads warp-uniform, values masked by lane)
                if (gi == 2) {
                    // max |v ek| first, times divi after the reduction: rounding is monotone,
                    // so this is the largest of the rounded products the fills below write
                    float mx = 0.f;
                    if (rset < NT)
                        for (int j = 0; j < nkr; j += 2) {
                            const int kc = j * H_KC + 16 * colq;
                            uint32_t v[32];
                            const bool two = j + 1 < nkr;     // uniform over the CTA
                            tmem_ld16_nw(lrow + 256u + 128u * rset + (uint32_t)kc, v);
                            if (two) tmem_ld16_nw(lrow + 256u + 128u * rset + (uint32_t)(kc + H_KC), v + 16);
#pragma unroll
                            for (int i = 16; i < 32; i++)
                                if (!two) v[i] = 0u;
                            tmem_wait16(v);
                            tmem_regs16(v + 16);
#pragma unroll
                            for (int g = 0; g < 2; g++) {
                                const int k0g = kc + g * H_KC;
                                const float4 *pq = reinterpret_cast<const float4 *>(s_p1f + (k0g & 127));
                                float q[16];
#pragma unroll
                                for (int u = 0; u < 4; u++) {
                                    const float4 f = pq[u];
                                    q[4 * u] = f.x, q[4 * u + 1] = f.y, q[4 * u + 2] = f.z, q[4 * u + 3] = f.w;
                                }
                                if (k0g + 16 <= nn) {
#pragma unroll
                                    for (int i = 0; i < 16; i++)
                                        mx = fmaxf(mx, fabsf(__uint_as_float(v[16 * g + i]) * fminf(q[i] + e2, radcut)));
                                } else {
#pragma unroll
                                    for (int i = 0; i < 16; i++)
                                        if (k0g + i < nn)
                                            mx = fmaxf(mx, fabsf(__uint_as_float(v[16 * g + i]) * fminf(q[i] + e2, radcut)));
                                }
                            }
                        }
                    if (rR >= n2) mx = 0.f;
                    mx *= divi;
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
                    if (lane == 0) atomicMax(&s_red[0], __float_as_uint(mx));
                    asm volatile("bar.sync 1, %0;" ::"n"(D2_FILL * 32) : "memory");
                    const float gm = __uint_as_float(s_red[0]);
                    int e = 0;
                    if (gm > 0.f) frexpf(gm, &e);       // gm < 2^e
                    const int se = min(100, max(-100, 12 - e));
                    sc2 = ldexpf(1.f, se);
                    s_exp += se;
                }
            }
            if (t >= H_NS) d2_wait(&empty[s], ph ^ 1, fail);
            const int k0 = jc * H_KC;
            if (gi == 0 && par == 0) {
                // B = Xs columns 2j + par, j in this chunk's 32 (rows r1), for both parities at
                // once: the chunk's 64 R columns are read once, the even columns split into
                // this stage's B and the odd ones into the next stage's (the par 1 chunk,
                // whose fill then only arrives), once the products that last read that stage
                // are complete.  Thread (row r, group kg of 8 j) reads 16 consecutive R
                // columns of its row from one 32-column tile
                const int s1 = s + 1 == H_NS ? 0 : s + 1, ph1 = s + 1 == H_NS ? ph ^ 1 : ph;
                if (t + 1 >= H_NS) d2_wait(&empty[s1], ph1 ^ 1, fail);
                // X tiles come with the par 0 chunks (t even) only: stage t % 3 took them
                // before at t - 6, t - 12, ..., so this is its phase t / 6
                d2_wait(&xfull[s], (t / 6) & 1, fail);
                const int e = threadIdx.x, rest = e >> 3, kg = rest & 3, r = (rest >> 2) * 8 + (e & 7);
                float v[8], v1[8];
                if (P.xt) {
                    // tile q = r / 32 holds rows R' < 64 of the chunk, column r % 32, under the
                    // 128-byte swizzle (16-byte granule ^ row % 8); R past npun2 (the next
                    // slab's rows, or the tensor's end) is zero
                    const unsigned char *tile = st + 16384 + (r >> 5) * 8192;
                    const int c = r & 31;
#pragma unroll
                    for (int i = 0; i < 8; i++) {
                        const int R = 16 * kg + 2 * i, R1 = R + 1;
                        const float x = *reinterpret_cast<const float *>(
                            tile + R * 128 + ((((c >> 2) ^ (R & 7)) << 4) | ((c & 3) << 2)));
                        const float x1 = *reinterpret_cast<const float *>(
                            tile + R1 * 128 + ((((c >> 2) ^ (R1 & 7)) << 4) | ((c & 3) << 2)));
                        v[i] = 64 * jc + R < n2 ? x * sx : 0.f;
                        v1[i] = 64 * jc + R1 < n2 ? x1 * sx : 0.f;
                    }
                } else {
                    const unsigned char *row = st + 16384 + (kg >> 1) * H_XT + r * 128;
                    const int q0 = (kg & 1) * 4;
#pragma unroll
                    for (int qq = 0; qq < 4; qq++) {
                        const float4 x = *reinterpret_cast<const float4 *>(row + (((q0 + qq) ^ (r & 7)) << 4));
                        v[2 * qq] = x.x * sx;
                        v[2 * qq + 1] = x.z * sx;
                        v1[2 * qq] = x.y * sx;
                        v1[2 * qq + 1] = x.w * sx;
                    }
                }
                if (r >= nn) {
#pragma unroll
                    for (int i = 0; i < 8; i++) v[i] = v1[i] = 0.f;
                }
                H_SPLIT8(small, H_SMALL_LO, kmaj16_off(r, 8 * kg), v, 0);
                H_SPLIT8(sm + (size_t)s1 * H_STAGE + H_SMALL_AT, H_SMALL_LO, kmaj16_off(r, 8 * kg), v1, 0);
            } else if (gi == 0) {
                // par 1: its B was split with the par 0 chunk (the fence below covers it)
            } else if (gi == 1) {
                // A = D1 rows R (sum or difference rows) from 16 E and O columns of lane i
                const int kc = k0 + 16 * colq;
                float ev[16], ov[16];
                tmem_ld16(lrow + (uint32_t)kc, ev);
                tmem_ld16(lrow + 128u + (uint32_t)kc, ov);
                if (on2) {
                    const bool fullc = kc + 16 <= nn;
#pragma unroll
                    for (int i = 0; i < 16; i++) {
                        const float x = (ev[i] + sg2 * ov[i]) * a13;
                        ev[i] = (fullc || kc + i < nn) ? x : 0.f;
                    }
                    H_SPLIT8(big, big_lo, kmaj16_off(R2, 16 * colq), ev, 0);
                    H_SPLIT8(big, big_lo, kmaj16_off(R2, 16 * colq + 8), ev, 8);
                }
            } else if (gi == 2) {
                // B = (D2 o F^T) rows R, 16 columns of R tile rset
                if (rset < NT) {
                    const int kc = k0 + 16 * colq;
                    float v[16];
                    tmem_ld16(lrow + 256u + 128u * rset + (uint32_t)kc, v);
                    const bool fullc = kc + 16 <= nn && rR < n2;
#pragma unroll
                    for (int i = 0; i < 16; i++) {
                        const float ek = fminf(s_p1f[kc + i] + e2, radcut);
                        const float x = v[i] * ek * divi * sc2;
                        v[i] = (fullc || (kc + i < nn && rR < n2)) ? x : 0.f;
                    }
                    H_SPLIT8(big, big_lo, kmaj16_off(rR, 16 * colq), v, 0);
                    H_SPLIT8(big, big_lo, kmaj16_off(rR, 16 * colq + 8), v, 8);
                }
            } else {
                // A = D3 columns 2j + par (rows r1): warp sub takes j in [k0 + 8 sub, +8)
                float v16[16];
                const int col0 = 2 * k0 + 16 * sub;
                tmem_ld16(lrow + (uint32_t)col0, v16);
                const bool fullc = col0 + 16 <= n2;
                float v[8];
#pragma unroll
                for (int uu = 0; uu < 8; uu++) {
                    const float x = (par == 0 ? v16[2 * uu] : v16[2 * uu + 1]) * a13;
                    v[uu] = (fullc || col0 + 2 * uu + par < n2) ? x : 0.f;
                }
                H_SPLIT8(small, H_SMALL_LO, kmaj16_off(m, 8 * sub), v, 0);
            }
            fence_async_smem();
            fence_before_sync();
            __syncwarp();
            if (lane == 0) mbar_arrive1(&full[s]);
            pt = s;
            pph = ph;
        });
        const int2 *srow = p.rows_ok[a] ? s_rows : nullptr;
        if (!srow) d2_prefetch_map(p, a, m, nn, h, sub);
        d2_wait(&empty[pt], pph, fail);
        fence_after_sync();
        if (!*fail) d2_store_h(p, a, p.foff[seg], m, nn, h, sub, lrow, ldexpf(1.f, -(4 * H_S_EXP + s_exp)), srow);
    }
    const int lt = total - 1, ls = lt % H_NS, lph = (lt / H_NS) & 1;
    if (lane == 0 && warp == D2_COPY_WARP && copies > 0) {
        const int c1 = copies - 1;
        mbar_wait(&full[c1 % H_NS], (c1 / H_NS) & 1);
    }
    if (lane == 0 && warp == D2_MMA_WARP) mbar_wait(&empty[ls], lph);
    fence_before_sync();
    __syncthreads();
    if (threadIdx.x == 0) {
        if (*fail) atomicExch(p.err, 1);
        P.xmax[seg] = 0u;                               // the next writer of X starts from zero
    }
    if (warp == 0) tmem_dealloc(tb, 512);
}

}  // namespace tc

namespace {

float tf32_round_nearest(float x)
{
    uint32_t u;
    std::memcpy(&u, &x, 4);
    u = (u + 0x1000u) & 0xFFFFE000u;      // nearest, ties away from zero (cvt.rna)
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}

// one n x n DST-I matrix (n <= 128) as K-chunks: each chunk [hi plane][lo plane]
// of 128 rows x D2_KC k in the canonical K-major layout, zero padded
void append_planes(std::vector<float> &out, const std::vector<double> &S, int n)
{
    size_t base = out.size();
    const size_t plane = (size_t)128 * tc::D2_KC;
    out.resize(base + (size_t)tc::D2_NKH * 2 * plane, 0.f);
    for (int r = 0; r < n; r++)
        for (int k = 0; k < n; k++) {
            float x = (float)S[(size_t)r * n + k], h = tf32_round_nearest(x), l = x - h;
            int c = k / tc::D2_KC, kk = k % tc::D2_KC;
            size_t o = (size_t)((r & 7) * 16 + (r >> 3) * tc::D2_SBO + (kk & 3) * 4 + (kk >> 2) * 128) / 4;
            out[base + (size_t)c * 2 * plane + o] = h;
            out[base + (size_t)c * 2 * plane + plane + o] = l;
        }
}

// S2 (n <= 256) folded by parity: [parity][chunk][hi, lo] with element
// (i, j) = S2[i][2j + parity] for i < ceil(n/2), zero padded to 128 x 128
std::vector<float> s2_fold_planes(const std::vector<double> &S, int n)
{
    const size_t plane = (size_t)128 * tc::D2_KC;
    std::vector<float> out((size_t)2 * tc::D2_NKH * 2 * plane, 0.f);
    const int h = (n + 1) / 2;
    for (int par = 0; par < 2; par++)
        for (int i = 0; i < h; i++)
            for (int j = 0; 2 * j + par < n; j++) {
                float x = (float)S[(size_t)i * n + 2 * j + par], hi = tf32_round_nearest(x), lo = x - hi;
                int c = j / tc::D2_KC, kk = j % tc::D2_KC;
                size_t o = (size_t)((i & 7) * 16 + (i >> 3) * tc::D2_SBO + (kk & 3) * 4 + (kk >> 2) * 128) / 4;
                size_t base = ((size_t)par * tc::D2_NKH + c) * 2 * plane;
                out[base + o] = hi;
                out[base + plane + o] = lo;
            }
    return out;
}

// the FP16 forms: x 2^12 split into hi = fp16(x) and lo = fp16(x - hi), chunks
// of 128 rows x 32 k in the canonical K-major layout of 16-bit values
inline void put16(std::vector<__half> &out, size_t base, int r, int k, double x)
{
    const double xs = x * (double)(1 << tc::H_S_EXP);
    const __half h = __double2half(xs);
    const __half l = __double2half(xs - (double)__half2float(h));
    const int c = k / tc::H_KC, kk = k % tc::H_KC;
    const size_t plane = (size_t)128 * tc::H_KC;
    const size_t o = (size_t)((r & 7) * 16 + (r >> 3) * tc::H_SBO + (kk & 7) * 2 + (kk >> 3) * 128) / 2;
    out[base + (size_t)c * 2 * plane + o] = h;
    out[base + (size_t)c * 2 * plane + plane + o] = l;
}

void append_planes16(std::vector<__half> &out, const std::vector<double> &S, int n)
{
    size_t base = out.size();
    out.resize(base + (size_t)tc::H_NKH * 2 * 128 * tc::H_KC, __float2half(0.f));
    for (int r = 0; r < n; r++)
        for (int k = 0; k < n; k++) put16(out, base, r, k, S[(size_t)r * n + k]);
}

std::vector<__half> s2_fold_planes16(const std::vector<double> &S, int n)
{
    const size_t per = (size_t)tc::H_NKH * 2 * 128 * tc::H_KC;
    std::vector<__half> out(2 * per, __float2half(0.f));
    const int h = (n + 1) / 2;
    for (int par = 0; par < 2; par++)
        for (int i = 0; i < h; i++)
            for (int j = 0; 2 * j + par < n; j++) put16(out, (size_t)par * per, i, j, S[(size_t)i * n + 2 * j + par]);
    return out;
}

template <typename V>
int upload_vec(Ctx &c, V **dst, const std::vector<V> &v)
{
    *dst = nullptr;
    size_t bytes = sizeof(V) * std::max<size_t>(v.size(), 1);
    cudaError_t e = cudaMalloc((void **)dst, bytes);
    if (e == cudaSuccess) {
        c.allocs.push_back(*dst);
        if (!v.empty()) e = cudaMemcpy(*dst, v.data(), sizeof(V) * v.size(), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) {
        c.err = std::string("fused DST tables: ") + cudaGetErrorString(e);
        return MW3_ERR_CUDA;
    }
    return MW3_OK;
}

}  // namespace

std::vector<double> dst_matrix(int n);

// Tables of the fused radial kernel; c.use_tc_dst2d stays false when the shape
// is outside it (npun2 > 256 or an r1 DST length above 128: the three-kernel
// tensor-core path or the CUDA-core path runs instead).
int build_tc_dst2d(Ctx &c)
{
    c.use_tc_dst2d = false;
    c.x_t = false;
    // n1 a multiple of 4: the kernel reads the r1 momenta as float4
    // n2 a multiple of 4: the rectangles' rows are a 16-byte multiple for the tensor copies
    if (c.fp64 || !c.use_tc || c.k_dst >= 2 || c.n2 > 256 || (c.n1 & 3) != 0 || (c.n2 & 3) != 0) return MW3_OK;
    const int na = c.na, W = (int)c.waves.size();
    for (auto &t : c.waves)
        for (int a = 0; a < na; a++)
            if (t.nopr1[a] > 128 || t.nopr1[a] < 1) return MW3_OK;
    std::vector<double> S2 = dst_matrix(c.n2);
    std::vector<float> fold = s2_fold_planes(S2, c.n2);
    std::vector<__half> fold16 = s2_fold_planes16(S2, c.n2), planes16;
    std::vector<float> planes;
    std::map<int, int64_t> off, off16;
    std::vector<int64_t> s1off((size_t)W * na), s1off16((size_t)W * na);
    // the r1 momenta padded by one chunk: the kernel reads them 16 at a time
    std::vector<float> p1f((size_t)W * na * c.n1 + 16, 0.f), p2f((size_t)W * na * c.n2);
    for (int w = 0; w < W; w++) {
        const WaveTables &t = c.waves[w];
        for (int a = 0; a < na; a++) {
            int nn = t.nopr1[a];
            auto it = off.find(nn);
            if (it == off.end()) {
                std::vector<double> S1 = dst_matrix(nn);
                int64_t o = (int64_t)planes.size();
                append_planes(planes, S1, nn);
                it = off.emplace(nn, o).first;
                int64_t o16 = (int64_t)planes16.size();
                append_planes16(planes16, S1, nn);
                off16.emplace(nn, o16);
            }
            s1off[(size_t)w * na + a] = it->second;
            s1off16[(size_t)w * na + a] = off16[nn];
        }
        for (size_t i = 0; i < t.p2r1.size(); i++) p1f[(size_t)w * na * c.n1 + i] = (float)t.p2r1[i];
        for (size_t i = 0; i < t.p2r2.size(); i++) p2f[(size_t)w * na * c.n2 + i] = (float)t.p2r2[i];
    }
    int rc;
    const char *tf = std::getenv("MW3_DST_TF32");
    c.dst_f16 = c.k_dst == 0 ? true : c.k_dst == 1 ? false : !(tf && tf[0] == '1');
    __half *p16 = nullptr, *f16 = nullptr;
    if ((rc = upload_vec(c, &p16, planes16))) return rc;
    if ((rc = upload_vec(c, &f16, fold16))) return rc;
    c.d_dst_planes16 = p16;
    c.d_dst_s2fold16 = f16;
    if ((rc = upload_vec(c, &c.d_dst_s1off16, s1off16))) return rc;
    if ((rc = upload_vec(c, &c.d_xmax, std::vector<unsigned>((size_t)c.G * na, 0u)))) return rc;
    if ((rc = upload_vec(c, &c.d_dst_planes, planes))) return rc;
    if ((rc = upload_vec(c, &c.d_dst_s2fold, fold))) return rc;
    if ((rc = upload_vec(c, &c.d_dst_s1off, s1off))) return rc;
    if ((rc = upload_vec(c, &c.d_p2r1f, p1f))) return rc;
    if ((rc = upload_vec(c, &c.d_p2r2f, p2f))) return rc;
    c.use_tc_dst2d = true;
    return MW3_OK;
}

bool xt_eligible(const Ctx &c)
{
    return c.use_tc_dst2d && c.dst_f16 && c.use_tc_ang && c.ec_nt == 0 && c.n1 % 4 == 0 && c.n1 >= 32;
}

int encode_tc_dst2d_xmap(Ctx &c)
{
    static_assert(sizeof(CUtensorMap) == sizeof(c.dst_xmap), "tensor map size");
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
        c.err = "cuTensorMapEncodeTiled is not available";
        return MW3_ERR_CUDA;
    }
    // [..][r1][R]: rows every r1 line of every slab, [G * na * n1], columns R, [n2], box
    // 32 x 128; transposed [..][R][r1] (MW3_X_T=1): rows every R line, [G * na * n2],
    // columns r1, [n1], box 32 x 64 (the first product's 64 R of a K chunk, 32 r1 a
    // box).  The transposed layout coalesces the update's rectangle stores (1.47 ->
    // 1.26 ms on the J = 0..40 sweep) but the angular kernel's tile copies, with the
    // lanes along r1, land 16 lanes on one shared-memory bank (2.05 -> 3.15 ms), so it
    // is not the default
    const char *xt = std::getenv("MW3_X_T");
    c.x_t = xt_eligible(c) && (c.k_xt == 1 || (c.k_xt < 0 && xt && xt[0] == '1'));
    const cuuint64_t dims[2] = {(cuuint64_t)(c.x_t ? c.n1 : c.n2),
                                (cuuint64_t)c.G * c.na * (c.x_t ? c.n2 : c.n1)};
    const cuuint64_t strides[1] = {(cuuint64_t)(c.x_t ? c.n1 : c.n2) * sizeof(float)};
    const cuuint32_t box[2] = {32, c.x_t ? 64u : 128u}, es[2] = {1, 1};
    CUtensorMap m;
    CUresult r = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn)(
        &m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, c.d_X, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
        CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        c.err = "cuTensorMapEncodeTiled failed for the rectangles";
        return MW3_ERR_CUDA;
    }
    std::memcpy(c.dst_xmap, &m, sizeof(m));
    return MW3_OK;
}

void launch_tc_dst2d(Ctx &c, const float *X, float *H, int g_begin, int g_end)
{
    using namespace tc;
    static bool attr = false;
    // stages, barriers and momenta, the row table (n2 <= 256), alignment slack
    const size_t smem = D2_BYTES + 1024 + 8192 + 1024;
    static_assert(H_BYTES == D2_BYTES, "both forms take the same shared memory");
    if (!attr) {
        cudaFuncSetAttribute(k_tc_dst2d, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(k_tc_dst2d_h, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = true;
    }
    int nseg = (g_end - g_begin) * c.na;
    if (nseg <= 0) return;
    Dst2Args p;
    p.X = X; p.H = H;
    p.s2fold = c.d_dst_s2fold; p.s1planes = c.d_dst_planes; p.s1off = c.d_dst_s1off; p.nopr1 = c.d_nopr1;
    p.p2r1f = c.d_p2r1f; p.p2r2f = c.d_p2r2f; p.radcut = (float)c.grid.radcutmax;
    p.mapT = c.d_mapT; p.foff = c.d_foff; p.blk_wave = c.d_blk_wave;
    p.rows = reinterpret_cast<const int2 *>(c.d_rows); p.rows_ok = c.d_rows_ok;
    static int nsm = 0;
    if (!nsm) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (nsm <= 0) nsm = 1;
    }
    p.wave = nsm;
    p.na = c.na; p.n1 = c.n1; p.n2 = c.n2; p.seg0 = g_begin * c.na;
    p.err = c.d_tc_err;
    CUtensorMap xmap;
    std::memcpy(&xmap, c.dst_xmap, sizeof(xmap));
    if (c.dst_f16) {
        Dst2hArgs P;
        P.b = p;
        P.s2fold = static_cast<const __half *>(c.d_dst_s2fold16);
        P.s1planes = static_cast<const __half *>(c.d_dst_planes16);
        P.b.s1off = c.d_dst_s1off16;
        P.xmax = c.d_xmax;
        P.xt = c.x_t ? 1 : 0;
        k_tc_dst2d_h<<<nseg, D2_WARPS * 32, smem, c.stream>>>(P, xmap);
    } else {
        k_tc_dst2d<<<nseg, D2_WARPS * 32, smem, c.stream>>>(p, xmap);
    }
    c.launches++;
}

}  // namespace mw3
