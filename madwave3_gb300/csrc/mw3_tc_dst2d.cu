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
    const int64_t *foff;
    const int *blk_wave;
    int na, n1, n2, seg0;
    int *err;
};

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
            // the r1 momenta of the slab into shared memory (read 8 at a time by the third product)
            const float *p1f = p.p2r1f + ((size_t)w * na + a) * n1;
            if (threadIdx.x < 128) s_p1f[threadIdx.x] = threadIdx.x < nn ? p1f[threadIdx.x] : 0.f;
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
        const int *mT = p.mapT + (size_t)a * n2 * n1;
        if (m < nn) {
            // the map entries this thread reads, into L1 while the last MMAs run
#pragma unroll 4
            for (int uu = 0; uu < 32; uu++) {
                int i = 32 * sub + uu;
                if (i < h) asm volatile("prefetch.global.L1 [%0];" ::"l"(mT + (size_t)i * n1 + m));
                if (i < n2 - h) asm volatile("prefetch.global.L1 [%0];" ::"l"(mT + (size_t)(n2 - 1 - i) * n1 + m));
            }
        }
        d2_wait(&empty[(total - 1) & (D2_NS - 1)], ((total - 1) >> 2) & 1, fail);
        fence_after_sync();
        if (!*fail) {
            const int64_t fo = p.foff[seg];
#pragma unroll
            for (int cc = 0; cc < 2; cc++) {
                const int i0 = 32 * sub + 16 * cc;
                float e[16], o[16];
                tmem_ld16(lrow + 256u + (uint32_t)i0, e);
                tmem_ld16(lrow + 384u + (uint32_t)i0, o);
                int is[16], id[16];
#pragma unroll
                for (int uu = 0; uu < 16; uu++) {
                    int i = i0 + uu;
                    is[uu] = (m < nn && i < h) ? __ldg(mT + (size_t)i * n1 + m) : -1;
                    id[uu] = (m < nn && i < n2 - h) ? __ldg(mT + (size_t)(n2 - 1 - i) * n1 + m) : -1;
                }
#pragma unroll
                for (int uu = 0; uu < 16; uu++) {
                    if (is[uu] >= 0) p.H[fo + is[uu]] = e[uu] + o[uu];
                    if (id[uu] >= 0) p.H[fo + id[uu]] = e[uu] - o[uu];
                }
            }
        }
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
    // n1 a multiple of 4: the kernel reads the r1 momenta as float4
    // n2 a multiple of 4: the rectangles' rows are a 16-byte multiple for the tensor copies
    if (c.fp64 || !c.use_tc || c.n2 > 256 || (c.n1 & 3) != 0 || (c.n2 & 3) != 0) return MW3_OK;
    const int na = c.na, W = (int)c.waves.size();
    for (auto &t : c.waves)
        for (int a = 0; a < na; a++)
            if (t.nopr1[a] > 128 || t.nopr1[a] < 1) return MW3_OK;
    std::vector<float> fold = s2_fold_planes(dst_matrix(c.n2), c.n2);
    std::vector<float> planes;
    std::map<int, int64_t> off;
    std::vector<int64_t> s1off((size_t)W * na);
    // the r1 momenta padded by one chunk: the kernel reads them 16 at a time
    std::vector<float> p1f((size_t)W * na * c.n1 + 16, 0.f), p2f((size_t)W * na * c.n2);
    for (int w = 0; w < W; w++) {
        const WaveTables &t = c.waves[w];
        for (int a = 0; a < na; a++) {
            int nn = t.nopr1[a];
            auto it = off.find(nn);
            if (it == off.end()) {
                int64_t o = (int64_t)planes.size();
                append_planes(planes, dst_matrix(nn), nn);
                it = off.emplace(nn, o).first;
            }
            s1off[(size_t)w * na + a] = it->second;
        }
        for (size_t i = 0; i < t.p2r1.size(); i++) p1f[(size_t)w * na * c.n1 + i] = (float)t.p2r1[i];
        for (size_t i = 0; i < t.p2r2.size(); i++) p2f[(size_t)w * na * c.n2 + i] = (float)t.p2r2[i];
    }
    int rc;
    if ((rc = upload_vec(c, &c.d_dst_planes, planes))) return rc;
    if ((rc = upload_vec(c, &c.d_dst_s2fold, fold))) return rc;
    if ((rc = upload_vec(c, &c.d_dst_s1off, s1off))) return rc;
    if ((rc = upload_vec(c, &c.d_p2r1f, p1f))) return rc;
    if ((rc = upload_vec(c, &c.d_p2r2f, p2f))) return rc;
    c.use_tc_dst2d = true;
    return MW3_OK;
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
    // rows: every r1 line of every slab, [G * na * n1]; columns: R, [n2]; box 32 x 128
    const cuuint64_t dims[2] = {(cuuint64_t)c.n2, (cuuint64_t)c.G * c.na * c.n1};
    const cuuint64_t strides[1] = {(cuuint64_t)c.n2 * sizeof(float)};
    const cuuint32_t box[2] = {32, 128}, es[2] = {1, 1};
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
    const size_t smem = D2_BYTES + 1024 + 1024;         // stages, barriers and momenta, alignment slack
    if (!attr) {
        cudaFuncSetAttribute(k_tc_dst2d, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = true;
    }
    int nseg = (g_end - g_begin) * c.na;
    if (nseg <= 0) return;
    Dst2Args p;
    p.X = X; p.H = H;
    p.s2fold = c.d_dst_s2fold; p.s1planes = c.d_dst_planes; p.s1off = c.d_dst_s1off; p.nopr1 = c.d_nopr1;
    p.p2r1f = c.d_p2r1f; p.p2r2f = c.d_p2r2f; p.radcut = (float)c.grid.radcutmax;
    p.mapT = c.d_mapT; p.foff = c.d_foff; p.blk_wave = c.d_blk_wave;
    p.na = c.na; p.n1 = c.n1; p.n2 = c.n2; p.seg0 = g_begin * c.na;
    p.err = c.d_tc_err;
    CUtensorMap xmap;
    std::memcpy(&xmap, c.dst_xmap, sizeof(xmap));
    k_tc_dst2d<<<nseg, D2_WARPS * 32, smem, c.stream>>>(p, xmap);
    c.launches++;
}

}  // namespace mw3
